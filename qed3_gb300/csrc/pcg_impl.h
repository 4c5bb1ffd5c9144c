// Preconditioned persistent CG (pcg.cu): host entry points.
#pragma once

#include <cuda_runtime.h>

#include "handles.h"
#include "lpc_impl.h"

namespace qed3 {
// sites per block of the register-resident solvers on `sm_count` SMs
int pcg_block_sites(int Ns, int sm_count);
bool pcg_plan(int prec, int nw, int Ns, int per, int sm_count, int* grid, int* threads, int* spt, size_t* smem);
int pcg_solve(qed3_dirac_s* d, qed3_lpc_s* L, double* x, const double* b, const qed3_solve_params* prm,
              qed3_solve_report* rep, cudaStream_t st);
}  // namespace qed3
