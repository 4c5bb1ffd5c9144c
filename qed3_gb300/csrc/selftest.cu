// Self-test of the bounded device waits.  Two blocks; block 1 never reaches
// the grid barriers, so block 0's waits can only end by running out: after
// spin_limit polls each barrier raises its abort flag and returns false.  The
// host reads the outcome; the context stays usable.  Exercises the exact
// barrier code of the persistent solvers (grid_sync2: register-resident CG,
// PCG; grid_sync: streaming CG) and the per-system step wait of the dynamic
// batched schedule (wait_step on an epoch nothing releases) without faulting
// or hanging anything.

#include "device.cuh"
#include "handles.h"

namespace qed3 {

__global__ void k_selftest_wait(GridBar2* bar2, GridBar* bar1, GridBar* bar3, const int* sys, long long spin_limit,
                                int* out) {
  if (blockIdx.x == 1) return;  // never arrives
  unsigned int epoch = 0, gen = 0;
  const bool ok2 = grid_sync2(bar2, epoch, spin_limit);
  const bool ok1 = grid_sync(bar1, gen, spin_limit);
  if (threadIdx.x == 0) {
    // a system in step 0 (sys[0] = epoch 0, sys[1] = state 0, not done) that nothing advances
    const int w = wait_step(sys, 1, sys + 1, 5, &bar3->abort, spin_limit);
    out[0] = ok2 ? 0 : 1;
    out[1] = ok1 ? 0 : 1;
    out[2] = ld_volatile_int(&bar2->abort);
    out[3] = ld_volatile_int(&bar1->abort);
    out[4] = (w == 2 && ld_volatile_int(&bar3->abort)) ? 1 : 0;
  }
}

int selftest_wait_timeout(long long spin_limit, int* timed_out_v2, int* timed_out_streaming) {
  if (spin_limit < 1 || spin_limit > 10000000LL) return fail(QED3_ERR_ARG, "spin_limit must be in [1, 1e7]");
  GridBar2* b2 = nullptr;
  GridBar* b1 = nullptr;
  GridBar* b3 = nullptr;
  int* sys = nullptr;
  int* out = nullptr;
  auto cleanup = [&]() {
    if (b2) cudaFree(b2);
    if (b1) cudaFree(b1);
    if (b3) cudaFree(b3);
    if (sys) cudaFree(sys);
    if (out) cudaFree(out);
  };
  if (cudaMalloc(&b2, sizeof(GridBar2)) != cudaSuccess || cudaMalloc(&b1, sizeof(GridBar)) != cudaSuccess ||
      cudaMalloc(&b3, sizeof(GridBar)) != cudaSuccess || cudaMalloc(&sys, 2 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&out, 5 * sizeof(int)) != cudaSuccess) {
    cleanup();
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  int h[5] = {0, 0, 0, 0, 0};
  cudaError_t e = cudaMemset(b2, 0, sizeof(GridBar2));
  if (e == cudaSuccess) e = cudaMemset(b1, 0, sizeof(GridBar));
  if (e == cudaSuccess) e = cudaMemset(b3, 0, sizeof(GridBar));
  if (e == cudaSuccess) e = cudaMemset(sys, 0, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(out, 0, 5 * sizeof(int));
  if (e == cudaSuccess) {
    k_selftest_wait<<<2, 32>>>(b2, b1, b3, sys, spin_limit, out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, out, sizeof(h), cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return fail(QED3_ERR_CUDA, std::string("self-test: ") + cudaGetErrorString(e));
  if (timed_out_v2) *timed_out_v2 = h[0] && h[2];
  // the streaming barrier and the batched step wait share the second flag
  if (timed_out_streaming) *timed_out_streaming = h[1] && h[3] && h[4];
  return (h[0] && h[1] && h[4]) ? QED3_ERR_TIMEOUT : QED3_OK;
}

}  // namespace qed3
