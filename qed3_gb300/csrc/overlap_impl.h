// Overlap driver (overlap.cpp).
#pragma once

#include <cuda_runtime.h>

#include "handles.h"

namespace qed3 {
int overlap_create(qed3_dirac_s* d, int order, int prec, qed3_overlap_s** out);
void overlap_destroy(qed3_overlap_s* ov);
int overlap_update(qed3_overlap_s* ov, double lmin, double lmax, double tol_outer, cudaStream_t st);
int overlap_apply(qed3_overlap_s* ov, int op, double* out, const double* in, double tol, qed3_solve_report* rep,
                  cudaStream_t st);
int overlap_force(qed3_overlap_s* ov, const double* eta, double* F, double tol, qed3_solve_report* rep,
                  cudaStream_t st);
int overlap_solve(qed3_overlap_s* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                  int flags, qed3_solve_report* rep, cudaStream_t st);
int overlap_project_low_modes(qed3_overlap_s* ov, int nev, double tol, int maxsteps, double margin,
                              cudaStream_t st);
int overlap_set_pole_solver(qed3_overlap_s* ov, int mode);
int overlap_set_mass(qed3_overlap_s* ov, double m);
int overlap_low_modes_info(const qed3_overlap_s* ov, int* nev, double* max_residual, int* lanczos_steps,
                           double* mu);
qed3_dirac_s* overlap_dirac(qed3_overlap_s* ov);
int overlap_info(const qed3_overlap_s* ov, double* lmin, double* lmax, double* k, double* delta, int* np,
                 int* np_fp64);
}  // namespace qed3
