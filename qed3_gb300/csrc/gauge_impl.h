// Host-side functions of gauge.cu.
#pragma once

#include <cuda_runtime.h>

#include "handles.h"

namespace qed3 {
int gauge_prepare(qed3_lattice_s* lat);
void gauge_free(qed3_lattice_s* lat);
int gauge_plaquettes(qed3_lattice_s* lat, const double* A, double* th, cudaStream_t st);
int gauge_plaquette_avg(qed3_lattice_s* lat, const double* A, double* theta, double* avg, cudaStream_t st);
int gauge_action(qed3_lattice_s* lat, const double* A, double beta, int compact, double* S, cudaStream_t st);
int gauge_force(qed3_lattice_s* lat, const double* A, double beta, int compact, int exact, double* F, cudaStream_t st);
int fermion_force(qed3_dirac_s* d, const double* eta_ref, double* F, cudaStream_t st);
// F_l = sum_m c_m (Re<DZ_m, dD Y_m> + Re<DY_m, dD Z_m>) + cw Re<eta, dD w>, internal-order fields
int overlap_force_links(qed3_dirac_s* d, int np, const double* c, double cw, const S64* Z, const S64* Y,
                        const S64* DZ, const S64* DY, const S64* eta, const S64* w, double* F, cudaStream_t st);
qed3_rng_s* rng_create(int n_links, int n_sites, int seed);
void rng_destroy(qed3_rng_s* r);
void rng_counts(const qed3_rng_s* r, size_t* n_links, size_t* n_sites);
void rng_gaussian_links(qed3_rng_s* r, double width, double* out);
void rng_gaussian_spinor(qed3_rng_s* r, double* out);
void rng_gaussian_sites(qed3_rng_s* r, double width, double* out);
double rng_uniform(qed3_rng_s* r);
int rng_save(const qed3_rng_s* r, const char* path);
int rng_load(qed3_rng_s* r, const char* path);
void rng_z2_spinor(qed3_rng_s* r, double* out);
int hmc_fermion(qed3_lattice_s* lat, qed3_dirac_s* d, qed3_rng_s* rng, double* A, double beta, int compact, int exact,
                double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double tol, int prec, int no_reject,
                int* accepted, double* dH_out, int* cg_iters, cudaStream_t st);
int hmc_overlap(qed3_lattice_s* lat, qed3_overlap_s* ov, qed3_rng_s* rng, double* A, double beta, int compact,
                int exact, double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double lmin, double lmax,
                double tol, double tol_inner, int no_reject, int* accepted, double* dH_out, int* cg_iters,
                cudaStream_t st);
int ext_plaquettes(qed3_lattice_s* lat, int Nt, const double* A, double* ths, double* tht, cudaStream_t st);
int ext_gauge_action(qed3_lattice_s* lat, int Nt, double at, double gsq, const double* A, double* S, cudaStream_t st);
int ext_gauge_force(qed3_lattice_s* lat, int Nt, double at, double gsq, const double* A, double* F, cudaStream_t st);
int ext_polyakov(qed3_lattice_s* lat, int Nt, const double* A, double* P, double* avg, cudaStream_t st);
int hmc_pure_gauge(qed3_lattice_s* lat, qed3_rng_s* rng, double* A, double beta, int compact, int exact, double tmax,
                   int nsteps, int no_reject, int* accepted, double* dH, cudaStream_t st);
}  // namespace qed3
