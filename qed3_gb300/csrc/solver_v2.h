// Register-resident persistent CG (solver_v2.cu): launch descriptor and host entry points.
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace qed3 {

struct CgV2Args {
  int Ns;
  const int* nbr;
  const M64* H;
  const M64* Hd;
  const double* diag;
  const M32* H32;
  const M32* Hd32;
  const float* diag32;
  const S64* b;
  S64* x;        // published solution (fp64)
  S64* t64;      // fp64 halo for reliable updates
  void* halo_r;  // gathered in phase A
  void* halo_t;  // gathered in phase B
  double* partials;
  GridBar2* bar;
  double* scal;
  double tol2, delta2, shift;
  int maxiter;
  long long spin_limit;
};

bool cg_v2_plan(int prec, int Ns, int sm_count, int* grid, int* threads, int* spt);
int cg_v2_launch(int prec, int spt, int grid, int threads, CgV2Args& a, cudaStream_t st);

}  // namespace qed3
