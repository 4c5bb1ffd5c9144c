// Host-side functions implemented in the .cu translation units.
#pragma once

#include <functional>

#include <cuda_runtime.h>

#include "handles.h"

namespace qed3 {

int lattice_upload(qed3_lattice_s* lat);
int lattice_free(qed3_lattice_s* lat);

int dirac_init_device(qed3_dirac_s* d);
int dirac_free_device(qed3_dirac_s* d);
int dirac_set_links(qed3_dirac_s* d, const double* A, int on_device, cudaStream_t st);
int dirac_set_coefficients(qed3_dirac_s* d, const double* hop, const double* diag);
// replace the geometry blocks and diagonal by Dirac1fonS2's (mass m)
int dirac_use_1f(qed3_dirac_s* d, double m);
int dirac_apply_ref(qed3_dirac_s* d, int op, double* out, const double* in, cudaStream_t st);
int dirac_apply_field(qed3_dirac_s* d, int op, int prec, void* out, const void* in, int nrhs, cudaStream_t st);
// fp32 field apply with caller-supplied hop blocks (same lattice and diagonal)
int dirac_apply32_blocks(qed3_dirac_s* d, const M32* H, void* out, const void* in, int nrhs, cudaStream_t st);
int field_import(qed3_dirac_s* d, int prec, void* field, const double* in_ref, int nrhs, cudaStream_t st);
int field_export(qed3_dirac_s* d, int prec, double* out_ref, const void* field, int nrhs, cudaStream_t st);
// solver import of b / |b| (|b| stored at *nrm; part: 64 doubles of scratch)
// and export of |b| x
int field_import_unit(qed3_dirac_s* d, S64* field, const double* in_ref, double* part, double* nrm, cudaStream_t st);
int field_export_scaled(qed3_dirac_s* d, double* out_ref, const S64* field, const double* nrm, cudaStream_t st);

int cg_solve(qed3_dirac_s* d, double* x, const double* b, const qed3_solve_params* prm, qed3_solve_report* rep,
             cudaStream_t st);
int solver_free(qed3_dirac_s* d);
// solver scratch of the operator (allocated on first use) and the common
// epilogue of the persistent solvers: report, export of the solution
int ensure_work(qed3_dirac_s* d);
int cg_finish(qed3_dirac_s* d, double* x, qed3_solve_report* rep, cudaStream_t st);
int spectral_bounds(qed3_dirac_s* d, double tol, int maxsteps, double* lmin, double* lmax, int* steps_used,
                    cudaStream_t st);
// extremal eigenvalues of a hermitian positive operator on nd doubles (Lanczos)
int lanczos_extremal(long long nd, const std::function<int(double*, const double*)>& apply, double tol, int maxsteps,
                     double* lmin, double* lmax, int* steps_used, cudaStream_t st);
int bicgstab_solve(qed3_dirac_s* d, int op, double* x, const double* b, const qed3_solve_params* prm, double eps,
                   qed3_solve_report* rep, cudaStream_t st);
int cg_solve_noalloc(qed3_dirac_s* d, double* x, const double* b, const qed3_solve_params* prm,
                     qed3_solve_report* rep, cudaStream_t st);

}  // namespace qed3
