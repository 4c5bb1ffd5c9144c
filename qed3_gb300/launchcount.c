/* Kernel-launch counter for the benchmark (not part of libqed3): a CUPTI
 * runtime-API callback counts cudaLaunchKernel / cudaLaunchCooperativeKernel /
 * cudaLaunchKernelExC calls between lc_start() and lc_stop(), and separately
 * those whose kernel symbol lies in this library's namespace (qed3::). */
#include <cupti.h>
#include <string.h>

static CUpti_SubscriberHandle g_sub;
static volatile long long g_ours = 0, g_all = 0;
static int g_on = 0;

static void CUPTIAPI on_api(void* user, CUpti_CallbackDomain dom, CUpti_CallbackId cbid, const void* data) {
  (void)user;
  const CUpti_CallbackData* d = (const CUpti_CallbackData*)data;
  if (dom != CUPTI_CB_DOMAIN_RUNTIME_API || d->callbackSite != CUPTI_API_ENTER) return;
  if (cbid != CUPTI_RUNTIME_TRACE_CBID_cudaLaunchKernel_v7000 &&
      cbid != CUPTI_RUNTIME_TRACE_CBID_cudaLaunchCooperativeKernel_v9000 &&
      cbid != CUPTI_RUNTIME_TRACE_CBID_cudaLaunchKernelExC_v11060 &&
      cbid != CUPTI_RUNTIME_TRACE_CBID_cudaLaunchKernelExC_ptsz_v11060)
    return;
  g_all++;
  const char* s = d->symbolName;
  if (s && (strstr(s, "4qed3") || strstr(s, "qed3::"))) g_ours++;
}

int lc_start(void) {
  if (g_on) return 0;
  if (cuptiSubscribe(&g_sub, (CUpti_CallbackFunc)on_api, NULL) != CUPTI_SUCCESS) return -1;
  if (cuptiEnableDomain(1, g_sub, CUPTI_CB_DOMAIN_RUNTIME_API) != CUPTI_SUCCESS) {
    cuptiUnsubscribe(g_sub);
    return -2;
  }
  g_ours = g_all = 0;
  g_on = 1;
  return 0;
}

int lc_stop(long long* ours, long long* all) {
  if (!g_on) return -1;
  cuptiUnsubscribe(g_sub);
  g_on = 0;
  *ours = g_ours;
  *all = g_all;
  return 0;
}
