// CG solve that allocates nothing: qed3_cg_solve_noalloc.
//
// Some callers cannot allocate device memory at solve time: hosts whose device
// memory is entirely owned by another allocator or pool (for example a
// framework's caching allocator, or a fixed MPS memory limit), so a
// cudaMalloc from this library would fail or steal from the pool, and
// multi-stream drivers for which cudaFree's implicit device-wide
// synchronisation would serialise every stream.  The regular qed3_cg_solve
// allocates its workspace on first use; this entry point instead runs the
// same persistent CG kernel on a scratch area that is a file-scope static
// device array, sized for at most QED3_NOALLOC_MAX_SITES sites.
//
// Properties a caller must know:
//  * The array is created when the library is loaded on a device and held by
//    every GPU that loads the library until the process exits
//    (QED3_NOALLOC_MAX_SITES x 10 fields x 32 B + ~5 KB = about 6.6 MB).
//  * The first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current.
//  * All calls share the one array, which keeps the previous call's contents;
//    the barrier state is cleared by every call and every field is
//    initialised by the kernel.  Calls whose executions overlap on the GPU
//    (several streams, several threads) race on the array: serialise them.
//  * No cudaMalloc, cudaFree, event creation or allocating library routine is
//    called; the solve report's time is host wall-clock.
//  * The call returns once the solve has finished: it reads the solve's
//    scalars back from the device to pick the solution buffer and to fill the
//    report.

#include <chrono>
#include <cmath>
#include <mutex>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"

namespace qed3 {

constexpr int kNoallocMaxSites = QED3_NOALLOC_MAX_SITES;
constexpr int kNoallocMaxBlocks = (kNoallocMaxSites + 255) / 256;
constexpr size_t kFieldBytes = size_t(kNoallocMaxSites) * 32;
// 10 fields, then partials [2][max blocks][4] doubles, the barrier, the scalars
constexpr size_t kPartialsOff = 10 * kFieldBytes;
constexpr size_t kBarOff = kPartialsOff + size_t(2) * kNoallocMaxBlocks * 4 * sizeof(double);
constexpr size_t kScalOff = kBarOff + 256;
constexpr size_t kScratchBytes = kScalOff + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

int cg_launch_on_scratch(int prec, qed3_dirac_s* d, S64* b, S64* xhi, S64* xhi2, S64* t64, void* r, void* p, void* t,
                         void* xlo, void* rh, void* th, double* partials, int max_blocks, GridBar* bar, double* scal,
                         double tol, double delta, int maxiter, double shift, cudaStream_t st);

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once).
int scratch_address(unsigned char** out) {
  int dev = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(QED3_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(QED3_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<unsigned char*>(ptr);
  }
  *out = g_addr[dev];
  return QED3_OK;
}
}  // namespace

int cg_solve_noalloc(qed3_dirac_s* d, double* x, const double* b, const qed3_solve_params* prm,
                     qed3_solve_report* rep, cudaStream_t st) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set (call qed3_dirac_set_links)");
  if (d->Ns > kNoallocMaxSites)
    return fail(QED3_ERR_ARG, "qed3_cg_solve_noalloc: lattice has " + std::to_string(d->Ns) +
                                  " sites; the allocation-free solve supports at most " +
                                  std::to_string(kNoallocMaxSites) + " (n_refine <= 32)");
  const int prec = prm ? prm->precision : QED3_PREC_F64;
  if (prec < QED3_PREC_F64 || prec > QED3_PREC_BF16) return fail(QED3_ERR_ARG, "unknown precision");
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  S64* f[10];
  for (int k = 0; k < 10; k++) f[k] = reinterpret_cast<S64*>(base + k * kFieldBytes);
  double* partials = reinterpret_cast<double*>(base + kPartialsOff);
  GridBar* bar = reinterpret_cast<GridBar*>(base + kBarOff);
  double* scal = reinterpret_cast<double*>(base + kScalOff);
  const double tol = prm && prm->tol > 0 ? prm->tol : 1e-10;
  const double delta = prm && prm->delta > 0 ? prm->delta : 0.1;
  const int maxiter = prm && prm->maxiter > 0 ? prm->maxiter : 100000;
  const double shift = prm ? prm->shift : 0.0;

  const auto t0 = std::chrono::steady_clock::now();
  if ((rc = field_import_unit(d, f[0], b, partials, scal + 6, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridBar), st));  // the barrier must start at zero
  rc = cg_launch_on_scratch(prec, d, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], partials,
                            kNoallocMaxBlocks, bar, scal, tol, delta, maxiter, shift, st);
  if (rc) return rc;
  double sc[6];
  QED3_CUDA_TRY(cudaMemcpyAsync(sc, scal, sizeof(sc), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  S64* xres = (sc[5] != 0.0) ? f[2] : f[1];
  if ((rc = field_export_scaled(d, x, xres, scal + 6, st))) return rc;
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  qed3_solve_report r{};
  r.status = int(sc[4]);
  r.iters = int(sc[2]);
  r.reliable_updates = int(sc[3]);
  r.true_rel_res = sc[1] > 0 ? std::sqrt(sc[0] / sc[1]) : 0.0;
  r.ms = ms;
  if (rep) *rep = r;
  if (r.status == QED3_ERR_TIMEOUT) return fail(QED3_ERR_TIMEOUT, "grid barrier timed out inside the CG kernel");
  return QED3_OK;
}

}  // namespace qed3
