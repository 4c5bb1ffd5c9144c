// Tensor-core channel mixing (tc.cu): workspace and host entry points.
#pragma once

#include <cuda_runtime.h>

#include "handles.h"

namespace qed3 {

// bf16 GEMM operands (h, Hd h, Ho h rows), weight-gradient partials, error flag
struct TcWork {
  void* Xh = nullptr;
  void* Xa = nullptr;
  void* Xb = nullptr;
  float* part = nullptr;
  int* err = nullptr;
  long long rows = 0;
  int nparts = 0, sms = 0;
  int ensure(long long rows_needed, int sm_count);
  void release();
};

// X* = bf16 rows of h (16 channels, [B][Ns][2][16] complex) and its in-block hops
int tc_hops(TcWork& w, const qed3_dirac_s* d, const M32* H, int per, int B, const float2* h, cudaStream_t st);
// out[rows][16 complex] = layer (adj: its adjoint) applied to the X* rows
int tc_mix(TcWork& w, long long rows, const float2* W, int adj, float* out, cudaStream_t st);
// Gw[3][16][16] += weight gradient from the X* rows and the output gradient G
int tc_wgrad(TcWork& w, long long rows, const float* G, int adj, float2* Gw, cudaStream_t st);
// QED3_ERR_TIMEOUT if a tensor-core kernel gave up waiting (and clears the flag)
int tc_check(TcWork& w, cudaStream_t st);

}  // namespace qed3
