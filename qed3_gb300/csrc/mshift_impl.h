// Multi-shift CG (mshift.cu): host entry points.
#pragma once

#include <cuda_runtime.h>

#include "handles.h"

namespace qed3 {
constexpr int kMsMaxShifts = 64;
// certify = false: when every shift converged in the kernel, skip the FP64
// true residuals (reps[m].true_rel_res = -1) and the defect correction
int mshift_solve(qed3_dirac_s* d, int ns, const double* shifts, const double* b_ref, double* x_ref, S64* X, S64* Pm,
                 double tol, int maxiter, qed3_solve_report* reps, float* ms_out, cudaStream_t st,
                 bool certify = true);
// |b - (q + s x)|^2 over nd doubles (complex pairs)
int ms_residual(long long nd, const double* q, const double* x, double s, const double* b, double* part, double* out,
                cudaStream_t st);
}  // namespace qed3
