/* qed3-gb300: C ABI of the GB300-native fermion hot path of qed3.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status and never throws.  Device vectors are complex128 interleaved
 * (re, im) with index 2*x + s (site-major, spin-minor) in the REFERENCE site
 * order -- the layout of the reference's CuC* vectors
 * (src/dual/valence.h:44-45).  Link fields are float64 per link in the
 * reference link order (links sorted (i<j), angle oriented i -> j,
 * src/both_3d/gauge_ext.h:45-49).  `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream).
 *
 * Threading: a handle is not safe for concurrent use from several threads;
 * distinct handles are independent.  Entry points that return a report
 * synchronise their stream; the others are stream-ordered and asynchronous.
 */
#ifndef QED3_GB300_H
#define QED3_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace CUDA_CHECK/CUBLAS_CHECK exceptions and asserts,
 *      src/dual/gpu_header.h:52-88) ---------------------------------------- */
#define QED3_OK 0
#define QED3_ERR_ARG 1      /* invalid argument or size */
#define QED3_ERR_CUDA 2     /* a CUDA runtime call failed */
#define QED3_ERR_NOCONV 3   /* solver hit maxiter / stagnated / NaN */
#define QED3_ERR_TIMEOUT 4  /* a device-side grid barrier gave up waiting */
#define QED3_ERR_STATE 5    /* handle used in the wrong state */
#define QED3_ERR_NOMEM 6    /* device allocation failed */

/* operators (replace LinOp compositions, src/dual/sparse_matrix.h:4-39,
 * src/both_3d/dirac_pf.h:66-92) */
#define QED3_OP_D 0
#define QED3_OP_DDAG 1
#define QED3_OP_DDAGD 2 /* D^dagger D: D first, then D^dagger */
#define QED3_OP_DDDAG 3 /* D D^dagger */

/* storage precisions of the device-internal fields */
#define QED3_PREC_F64 0
#define QED3_PREC_F32 1
#define QED3_PREC_BF16 2 /* bf16-stored spinors, fp32 links and arithmetic */

typedef struct qed3_lattice_s qed3_lattice;
typedef struct qed3_dirac_s qed3_dirac;
typedef struct qed3_overlap_s qed3_overlap;
typedef struct qed3_lpc_s qed3_lpc;

/* Message of the last failure on the calling thread ("" if none). */
const char* qed3_last_error_string(void);
int qed3_version(void);
/* Self-test of the bounded device waits every persistent solver relies on:
 * a two-block launch in which one block never arrives at the grid barriers,
 * so the other's waits end only by running out after spin_limit polls (both
 * barrier forms: the register-resident solvers' and the streaming solver's).
 * Returns QED3_ERR_TIMEOUT when both waits ran out and raised their abort
 * flags (the expected outcome), QED3_OK otherwise; the CUDA context stays
 * usable.  No counterpart in the reference. */
int qed3_selftest_wait_timeout(long long spin_limit, int* timed_out_resident, int* timed_out_streaming);

/* ======================================================================
 * Lattice  --  replaces S2Trivalent(n_refine) (src/both_3d/s2n_dual.h:49-106)
 * and SpinStructureDual (src/both_3d/dirac_dual.h:15-60), which read the
 * offline generator's .dat tables (integrator/get_geometry.cc:383-465,
 * integrator/test_sorting.cc:430-594).  Built in O(N) on the host; tables are
 * uploaded to the current device in a space-filling-curve order.
 * ====================================================================== */
int qed3_lattice_create(int n_refine, qed3_lattice** out);
int qed3_lattice_destroy(qed3_lattice* lat);
/* n_sites = 20n^2, n_links = 30n^2, n_faces = 10n^2+2, face_total = sum |face| */
int qed3_lattice_sizes(const qed3_lattice* lat, int* n_sites, int* n_links, int* n_faces, int* face_total);
/* Host copies of the tables in reference order; any pointer may be NULL.
 * sites[Ns*3], nns[Ns*3], links[Nl*2], simp_links[Nl*2] (S2Trivalent::dual_links),
 * face_offsets[Nf+1], face_sites[face_total], ell[Nl], link_volume[Nl],
 * vols[Nf] (dual-face areas), omega[Nl] (omega(links[l][0], links[l][1])),
 * alpha[Ns*3] (alpha(x, nns[x][k])), means[3] = {mean_ell, mean_link_volume, mean_vol}. */
int qed3_lattice_tables(const qed3_lattice* lat, double* sites, int* nns, int* links, int* simp_links,
                        int* face_offsets, int* face_sites, double* ell, double* link_volume, double* vols,
                        double* omega, double* alpha, double* means);
/* Internal (device) order: perm[i] = reference index of internal site i. */
int qed3_lattice_permutation(const qed3_lattice* lat, int* perm);
/* The lattice of a caller's own simplicial mesh, so that sites and links carry
 * the caller's numbering -- e.g. the reference's S2Simp tables
 * (src/both_3d/s2n_simp.h:43-269: vertices, triangles) and S2Trivalent link
 * list (src/both_3d/s2n_dual.h:49-106), whose link angles a saved gauge
 * configuration is indexed by.  vertices[n_vertices*3] (normalised here),
 * triangles[n_triangles*3] (vertex ids, any winding); dual site t is the
 * circumcentre of triangle t.  links: NULL (lexicographic (i<j) order) or
 * [n_links*2] pairs giving the link numbering and orientation: link l points
 * links[l][0] -> links[l][1] (its angle enters the hop in that direction with
 * +A, as the reference's map2sign), in either label order.  The mesh must be a
 * closed triangulation of the sphere (every edge in two triangles, one ring
 * of triangles per vertex, V - E + F = 2); QED3_ERR_ARG otherwise. */
int qed3_lattice_from_mesh(int n_vertices, const double* vertices, int n_triangles, const int* triangles,
                           const int* links, qed3_lattice** out);
/* The simplicial mesh of a lattice: vertices[n_faces*3], triangles[n_sites*3]. */
int qed3_lattice_mesh(const qed3_lattice* lat, double* vertices, int* triangles);
/* Replaces the lattice's spin connection by a caller's tables, e.g. the
 * reference's SpinStructureDual files (src/both_3d/dirac_dual.h:15-60, written
 * by integrator/test_sorting.cc:430-594): omega[n_links] = omega(links[l][0],
 * links[l][1]), alpha[n_sites*3] = alpha(x, nns[x][k]) in this lattice's
 * numbering.  Either pointer may be NULL (that table is kept).  Operators
 * created afterwards (qed3_dirac_create) use them. */
int qed3_lattice_set_spin_structure(qed3_lattice* lat, const double* omega, const double* alpha);

/* ======================================================================
 * Wilson-Dirac operator  --  replaces DiracS2Dual / DiracExt<.., DiracS2Dual>
 * at Nt=1 (src/both_3d/dirac_dual.h:63-215, src/both_3d/dirac_ext.h:6-334)
 * together with its device form DWDevice + CSR (src/both_3d/sparse_dirac.h:5-166).
 * (D psi)_x = [M5 + sum_y r kappa_l/2] psi_x
 *           + sum_y kappa_l/2 (-r + gamma_xy) e^{i A_xy} Omega_xy psi_y
 * ====================================================================== */
int qed3_dirac_create(qed3_lattice* lat, double r, double M5, qed3_dirac** out);
/* Dirac1fonS2 (src/dual/dirac.h:145-220) on the same layout: hop blocks
 * -(vol_x/vbar)(r u_{x,k} - v_{x,k}.sigma) Omega e^{iU}, diagonal
 * sum_k (vol_x/vbar)(r u_{x,k} + m/3) + M5, with the u, v tables of
 * integrator/test_sorting.cc:499-594 computed from the lattice (vol_x: area of
 * x's triangle).  Every other call (set_links, apply, solvers, force) is the
 * same as for qed3_dirac_create's operator. */
int qed3_dirac_create_1f(qed3_lattice* lat, double r, double m, double M5, qed3_dirac** out);
int qed3_dirac_destroy(qed3_dirac* d);
/* DWDevice::update(U) (src/both_3d/sparse_dirac.h:144-151): rebuild every hop
 * matrix on the device from link angles A[n_links] (host or device pointer). */
int qed3_dirac_set_links(qed3_dirac* d, const double* A, int A_on_device, void* stream);
/* Load arbitrary coefficients of the same sparsity (any builder, e.g.
 * Dirac1fonS2::coo_format, src/dual/dirac.h:187-220): host hop[Ns*3*8] =
 * 2x2 complex row-major block of D at (x, nns[x][k]); host diag[Ns] = real
 * scalar of the diagonal block. */
int qed3_dirac_set_coefficients(qed3_dirac* d, const double* hop, const double* diag);
/* LinOp::operator()/Async (src/dual/sparse_matrix.h:4-39): out = op(in) on
 * device complex128 vectors of length 2*n_sites in reference order. */
int qed3_dirac_apply(qed3_dirac* d, int op, double* out, const double* in, void* stream);

/* Device-internal fields (space-filling-curve order, precision `prec`):
 * F64 = 32 B/site, F32 = 16 B/site, BF16 = 8 B/site, nrhs fields back to back.
 * These are what the solvers use; the reference-order calls above convert. */
size_t qed3_field_bytes(const qed3_dirac* d, int prec, int nrhs);
int qed3_field_import(qed3_dirac* d, int prec, void* field, const double* in_ref, int nrhs, void* stream);
int qed3_field_export(qed3_dirac* d, int prec, double* out_ref, const void* field, int nrhs, void* stream);
int qed3_dirac_apply_field(qed3_dirac* d, int op, int prec, void* out, const void* in, int nrhs, void* stream);

/* ======================================================================
 * Solvers  --  replace MatPoly::solve<N> (src/dual/matpoly.h:204-267):
 * CG on (D^dagger D + shift) x = b from x0 = 0.
 * ====================================================================== */
#define QED3_SOLVE_STREAMING 2 /* force the memory-streaming persistent kernel (default: register-resident when it fits) */
#define QED3_SOLVE_BCAST_B 4   /* batched: every right-hand side of system u is b[u]'s first vector */
#define QED3_SOLVE_FLEXIBLE 8  /* preconditioned CG: Polak-Ribiere beta = <z', r' - r> / <z, r> (flexible CG) */
#define QED3_SOLVE_PIPELINED 16 /* preconditioned CG: pipelined one-barrier recurrence (QED3_PREC_F32 only) */

typedef struct {
  double tol;     /* target ||b - A x|| / ||b|| of the FP64 true residual */
  int maxiter;    /* iteration cap (0 => 100000) */
  int precision;  /* QED3_PREC_F64: plain FP64 CG; F32/BF16: mixed precision with FP64 reliable updates */
  double delta;   /* reliable-update trigger: update when |r| < delta * max|r| since the last one (0 => 0.1) */
  double shift;   /* solve (D^dagger D + shift) x = b */
  int flags;
} qed3_solve_params;

typedef struct {
  int status;          /* QED3_OK or QED3_ERR_NOCONV / _TIMEOUT */
  int iters;           /* CG iterations */
  int reliable_updates;
  double true_rel_res; /* ||b - A x|| / ||b|| recomputed in FP64 on the device */
  double ms;           /* device time of the solve */
} qed3_solve_report;

/* x, b: device complex128, reference order.  report may be NULL (then the
 * call is asynchronous and the outcome is read with qed3_solver_last_report). */
int qed3_cg_solve(qed3_dirac* d, double* x, const double* b, const qed3_solve_params* params,
                  qed3_solve_report* report, void* stream);
int qed3_solver_last_report(qed3_dirac* d, qed3_solve_report* report);

/* Extremal eigenvalues of D^dag D by FP64 Lanczos on the device -- an
 * alternative to the power / inverse-power iterations of
 * Overlap::compute_lambda_max (src/both_3d/overlap.h:217-306) that needs no
 * solves.  Stops when both extremal Ritz values change by less than tol
 * (relative) over two consecutive checks (every max(10, m/16) steps at step
 * m); returns QED3_ERR_NOCONV (with
 * the last estimates) after maxsteps.  Ritz values lie inside the spectrum:
 * lambda_min is approached from above, lambda_max from below. */
int qed3_dirac_spectral_bounds(qed3_dirac* d, double tol, int maxsteps, double* lambda_min, double* lambda_max,
                               int* steps, void* stream);

/* BiCGStab with restarts  --  replaces MatPoly::bicgstab
 * (src/dual/matpoly.h:366-479), which the reference keeps for experiments.
 * Solves (op + shift) x = b for op = QED3_OP_D, _DDAG or _DDAGD (device
 * complex128, reference order) in FP64 (params->precision must be
 * QED3_PREC_F64), with the reference's start x0 = b, its stopping rules
 * (|r|^2 < tol^2 |r0|^2, or |t|^2 < eps absolute) and restarts
 * (|<rc,r>| < eps).  eps < 0 selects the reference default 1e-8.  The
 * report's true_rel_res is ||b - (op + shift) x|| / ||b||. */
int qed3_bicgstab_solve(qed3_dirac* d, int op, double* x, const double* b, const qed3_solve_params* params,
                        double eps, qed3_solve_report* report, void* stream);

/* Allocation-free CG solve.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory at solve time -- hosts whose
 * device memory is owned by another allocator or pool, multi-stream drivers
 * that must avoid cudaFree's device-wide synchronisation.  Same algorithm, arguments and report as
 * qed3_cg_solve, but its scratch is a static device array of the library
 * (about 6.6 MB, held by every GPU that loads the library until exit), so
 * lattices are limited to QED3_NOALLOC_MAX_SITES sites (n_refine <= 32);
 * larger ones return QED3_ERR_ARG.  The first call on a device looks up the
 * array's address.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised. */
#define QED3_NOALLOC_MAX_SITES 20480
int qed3_cg_solve_noalloc(qed3_dirac* d, double* x, const double* b, const qed3_solve_params* params,
                          qed3_solve_report* report, void* stream);

/* ======================================================================
 * S^2 x S^1: Nt time slices  --  replaces DiracExt<Lattice, DiracS2Dual>
 * (src/both_3d/dirac_ext.h:6-334) for Nt > 1: per slice the dual-lattice
 * hops with that slice's link angles, spin-diagonal temporal hops with
 * kappa_t = (triangle area) / mean_ell / at and antiperiodic time boundary,
 * diagonal M5 + sum r kappa / 2 + r kappa_t.  Vectors: complex128
 * [Nt][Ns][2] (index Nx s + 2 x + spin, Nx = 2 Ns); link angles on the
 * device: A[Nt][n_links] spatial, then A[Nt][n_sites] temporal (GaugeExt).
 * At Nt = 1 it is the dual-lattice operator.
 * ====================================================================== */
typedef struct qed3_dirac_ext_s qed3_dirac_ext;
int qed3_dirac_ext_create(qed3_lattice* lat, double r, double M5, int Nt, double at, qed3_dirac_ext** out);
int qed3_dirac_ext_destroy(qed3_dirac_ext* e);
int qed3_dirac_ext_set_links(qed3_dirac_ext* e, const double* A, void* stream);
/* op: QED3_OP_D, _DDAG, _DDAGD, _DDDAG; in may equal out for D and D^dag */
int qed3_dirac_ext_apply(qed3_dirac_ext* e, int op, double* out, const double* in, void* stream);
/* Fermion force F = -2 Re <D eta, dD/dA eta> for every spatial and temporal
 * link (DiracExt::d_coo_format, src/both_3d/dirac_ext.h:234-320), F in the
 * link layout; eta device complex128 [Nt][Ns][2]. */
int qed3_dirac_ext_fermion_force(qed3_dirac_ext* e, const double* eta, double* F, void* stream);
/* Point-source propagator (src/both_3d/prop.cu:243-268): sink = D^{-1} src1
 * with src1 = 1 at (slice s, site ix of the reference numbering, spin a),
 * solved as (D^dag D)^{-1} D^dag src1 by the CG (params->tol, ->precision
 * F64 or F32 as for qed3_dirac_ext_cg_solve; shift ignored); dagger != 0 (prop.cu's IS_DAGGER): sink = D^{-dag} src1
 * = (D D^dag)^{-1} D src1.  sink: device complex128 [Nt][n_sites][2]; synchronous. */
int qed3_dirac_ext_propagator(qed3_dirac_ext* e, int s, int ix, int a, int dagger, double* sink, const qed3_solve_params* params,
                              qed3_solve_report* report, void* stream);
/* Overlap<DiracExt> (src/both_3d/overlap.h:137-390 on this operator, the
 * reference's IS_OVERLAP builds of hmc.cu / prop.cu): Zolotarev order `order`,
 * all poles from one FP64 multi-shift CG on D^dag D.  update: lambda_min /
 * lambda_max given, or (both 0) from Lanczos on D^dag D to tol widened by the
 * relative margin.  apply: op = QED3_OP_D (D_ov), _DDAG (D_ov^dag), _DDAGD or
 * _DDDAG (D_ov + D_ov^dag = D_ov^dag D_ov); pole solves to tol_inner.  solve:
 * CG on D_ov^dag D_ov to tol (certified by the recomputed residual); prop != 0
 * solves for D_ov^dag b instead of b (prop.cu: sink = D_ov^{-1} b). */
typedef struct qed3_overlap_ext_s qed3_overlap_ext;
int qed3_overlap_ext_create(qed3_dirac_ext* e, int order, qed3_overlap_ext** out);
int qed3_overlap_ext_destroy(qed3_overlap_ext* ov);
int qed3_overlap_ext_update(qed3_overlap_ext* ov, double lambda_min, double lambda_max, double tol, double margin,
                            void* stream);
int qed3_overlap_ext_info(const qed3_overlap_ext* ov, double* lambda_min, double* lambda_max, double* k,
                          double* delta);
int qed3_overlap_ext_apply(qed3_overlap_ext* ov, int op, double* out, const double* in, double tol_inner,
                           int* pole_iters, void* stream);
int qed3_overlap_ext_solve(qed3_overlap_ext* ov, double* x, const double* b, double tol, double tol_inner,
                           int maxiter, int prop, qed3_solve_report* report, void* stream);
/* Overlap pseudofermion force, F = -2 d/dA Re<eta, D_ov eta> for every spatial
 * and temporal link (Overlap::precalc_grad + grad_deviceAsyncLaunch,
 * src/both_3d/overlap.h:393-470), pole solves to tol_inner. */
int qed3_overlap_ext_force(qed3_overlap_ext* ov, const double* eta, double* F, double tol_inner, void* stream);
/* MatPoly::solve on D^dag D (+ params->shift), certified by the FP64 true
 * residual.  params->precision QED3_PREC_F64: the reference's FP64 recurrence;
 * QED3_PREC_F32: FP32 iterations (FP32 copy of the operator) with FP64
 * reliable updates whenever the residual has dropped by params->delta. */
int qed3_dirac_ext_cg_solve(qed3_dirac_ext* e, double* x, const double* b, const qed3_solve_params* params,
                            qed3_solve_report* report, void* stream);

/* S^2 x S^1 gauge side: U1WilsonExt (src/both_3d/action_ext.h:4-161) and the
 * Polyakov loop (src/both_3d/obs.h:4-10).  A: device [Nt][n_links] spatial,
 * then [Nt][n_sites] temporal.  theta_s [Nt][n_faces] (spatial plaquettes),
 * theta_t [Nt][n_links] (temporal: A_s + A_t(s,y) - A_{s+1} - A_t(s,x)); the
 * action sum beta_s theta_s^2/2 + beta_t theta_t^2/2 with beta_s = at / vols / gsq,
 * beta_t = 2 / at * link_volume / ell^2 / gsq; F has A's layout; P[n_sites]
 * complex = exp(i sum_s A_t(s,x)), avg[2] its mean (either may be NULL). */
int qed3_ext_plaquettes(qed3_lattice* lat, int Nt, const double* A, double* theta_s, double* theta_t, void* stream);
int qed3_ext_gauge_action(qed3_lattice* lat, int Nt, double at, double gsq, const double* A, double* S, void* stream);
int qed3_ext_gauge_force(qed3_lattice* lat, int Nt, double at, double gsq, const double* A, double* F, void* stream);
int qed3_ext_polyakov(qed3_lattice* lat, int Nt, const double* A, double* P, double* avg, void* stream);

/* ======================================================================
 * Batched solves in ONE persistent launch  --  replaces the reference's
 * loops of MatPoly::solve over pseudofermions and Zolotarev poles on OpenMP
 * threads and CUDA streams (src/both_3d/overlap.h:309-332,
 * src/both_3d/hmc.h:172-200).  System u solves (D_u^dag D_u + shift) x = b
 * for nrhs[u] right-hand sides; systems may live on different lattices.
 * rhs_tile (right-hand sides sharing each stencil read: 1, 2, 4, 8 held in
 * one thread's registers; 16, 32 spread over consecutive threads of a warp)
 * and threads (128, 256) are chosen by the built-in autotuner when passed as 0.
 * ====================================================================== */
typedef struct qed3_batch_s qed3_batch;
int qed3_batch_create(int nsys, qed3_dirac* const* ops, const int* nrhs, int precision, int rhs_tile, int threads,
                      qed3_batch** out);
/* schedule of the persistent launch: QED3_BATCH_STATIC gives each system a
 * fixed range of blocks (re-split after every synchronous solve in proportion
 * to the iterations it took); QED3_BATCH_DYNAMIC cuts every system into tiles
 * of `threads` sites and hands the tiles of each CG step to whichever block is
 * free.  0: chosen by the autotuner with the tile and threads (static when
 * both of those are given). */
#define QED3_BATCH_STATIC 1
#define QED3_BATCH_DYNAMIC 2
int qed3_batch_create2(int nsys, qed3_dirac* const* ops, const int* nrhs, int precision, int rhs_tile, int threads,
                       int schedule, qed3_batch** out);
int qed3_batch_schedule(const qed3_batch* bt, int* schedule);
int qed3_batch_destroy(qed3_batch* bt);
/* tile and threads the batch runs with */
int qed3_batch_config(const qed3_batch* bt, int* rhs_tile, int* threads, int* blocks);
/* x[u], b[u]: device complex128, nrhs[u] vectors back to back (reference order);
 * shifts[u]: host [nrhs[u]] or NULL (then params->shift); reports: host
 * [sum nrhs] in system order, may be NULL; ms: device time of the launch. */
int qed3_batch_solve(qed3_batch* bt, double* const* x, const double* const* b, const double* const* shifts,
                     const qed3_solve_params* params, qed3_solve_report* reports, float* ms, void* stream);
/* The same solve split for CUDA-graph capture.  qed3_batch_set_shifts stores
 * the shifts (host [nrhs[u]] per system or NULL, then `shift`) on the device;
 * it copies only when a shift changed and refuses to copy while `stream` is
 * capturing.  qed3_batch_launch enqueues the gather of b, the persistent
 * launch and the scatter of x with no host synchronisation, allocation or
 * host-to-device copy, so the sequence can be captured and replayed (a replay
 * reuses the x, b pointers and shifts of the capture).  qed3_batch_reports
 * waits for `stream` and reports the last completed launch (ms = 0). */
int qed3_batch_set_shifts(qed3_batch* bt, const double* const* shifts, double shift, void* stream);
int qed3_batch_launch(qed3_batch* bt, double* const* x, const double* const* b, const qed3_solve_params* params,
                      void* stream);
int qed3_batch_reports(qed3_batch* bt, qed3_solve_report* reports, void* stream);

/* ======================================================================
 * Gauge side  --  replaces U1onS2::plaquette_angle/average_plaquette
 * (src/dual/gauge.h:90-110) and U1Wilson::operator()/get_force
 * (src/both/action.h:21-48, weights mean_vol/vol_f) on the dual faces.
 * A, theta, F are device float64 arrays (links / faces in reference order).
 * compact: 1 = -beta sum w cos(theta), 0 = beta/2 sum w theta^2.
 * exact: 1 = compact force with sin(theta); 0 = the reference's theta
 * (src/dual/action.h:37).
 * ====================================================================== */
int qed3_plaquette(qed3_lattice* lat, const double* A, double* theta, double* avg, void* stream);
int qed3_gauge_action(qed3_lattice* lat, const double* A, double beta, int compact, double* S, void* stream);
int qed3_gauge_force(qed3_lattice* lat, const double* A, double beta, int compact, int exact, double* F, void* stream);

/* Wilson fermion force of every link at once: F[l] = -2 Re <D eta, dD/dA_l eta>
 * (DiracPf::grad_deviceAsyncLaunch, src/both_3d/dirac_pf.h:107-122, which is
 * called once per link).  eta: device complex128, reference order; F: device [n_links]. */
int qed3_fermion_force(qed3_dirac* d, const double* eta, double* F, void* stream);

/* ======================================================================
 * RNG and pure-gauge HMC  --  ParallelRng2 (src/both/rng.h:76-125) driven by
 * libstdc++ mt19937_64 + normal_distribution, and HMCPureGauge::run
 * (src/both_3d/hmc.h:212-296).  dH is accumulated from per-term differences.
 * ====================================================================== */
typedef struct qed3_rng_s qed3_rng;
int qed3_rng_create(int n_links, int n_sites, int seed, qed3_rng** out);
int qed3_rng_destroy(qed3_rng* r);
/* Random-stream checkpoint in the reference's layout (ParallelRngExt::ckpoint
 * / read, src/both_3d/rng.h:131-168, at Nt = 1): a run saved by either side
 * continues with identical streams on the other. */
int qed3_rng_save(const qed3_rng* r, const char* path);
/* ParallelRng::uniform: one draw of the master engine (the Metropolis test). */
int qed3_rng_uniform(qed3_rng* r, double* out);
int qed3_rng_load(qed3_rng* r, const char* path);
/* Gauge checkpoint in the reference's layout (GaugeExt::ckpoint / read,
 * src/both_3d/gauge_ext.h:225-275, at Nt = 1): host A[n_links] in this
 * lattice's link numbering, then n_sites temporal angles (written as zero;
 * their largest magnitude is reported on load, since this path has no
 * temporal links). */
int qed3_links_save(const qed3_lattice* lat, const double* A, const char* path);
int qed3_links_load(const qed3_lattice* lat, double* A, double* temporal_max_abs, const char* path);
/* host outputs: links[n_links] = width * N(0,1); spinor[2*n_sites] complex
 * (ParallelRngExt::fill_gaussian, src/both_3d/rng.h:122-129) */
int qed3_rng_gaussian_links(qed3_rng* r, double width, double* links);
int qed3_rng_gaussian_spinor(qed3_rng* r, double* spinor);
/* FermionVector::set_random (src/dual/valence.h:54-60): host spinor[2*n_sites]
 * complex = (z + i z')/sqrt(2 n_sites) with z, z' = z2_site(x), which the
 * reference draws from uniform_int_distribution(1, 2). */
int qed3_rng_z2_spinor(qed3_rng* r, double* spinor);
/* FermionVector::set_pt_source (src/dual/valence.h:47-52): host spinor[2*n_sites]
 * complex = unit vector at (site x, spin s), reference order. */
int qed3_point_source(int n_sites, int x, int s, double* spinor);
/* HMC::run with one PseudoFermion (npf = 1) or HMC2::run with npf of them,
 * and ExplicitLeapfrogML (src/both_3d/hmc.h:75-110 and :172-200,
 * src/both_3d/pseudofermion.h:33-60, src/both_3d/integrator.h:58-168): one
 * trajectory of Wilson fermions + gauge action on the device, in place on the
 * device links A[n_links]; d is the operator (its links are set from A and,
 * on rejection, restored).  nsteps outer (fermion) steps of tmax/nsteps, each
 * with nsteps_inner gauge steps; pseudofermion solves to tol in `precision`,
 * certified by the FP64 true residual.  Writes accepted, dH, cg_iters. */
#define QED3_INTEGRATOR_LEAPFROG_ML 0 /* ExplicitLeapfrogML, src/both_3d/integrator.h:58-168 */
#define QED3_INTEGRATOR_LEAPFROG 1    /* ExplicitLeapfrog, src/dual/integrator.h:9-53 (nsteps_inner unused) */
int qed3_hmc_fermion(qed3_lattice* lat, qed3_dirac* d, qed3_rng* rng, double* A, double beta, int compact, int exact,
                     double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double tol, int precision,
                     int no_reject, int* accepted, double* dH, int* cg_iters, void* stream);
/* The same trajectory with overlap fermions (the reference's IS_OVERLAP build
 * of HMC2, src/both_3d/hmc.cu:155-160,457-467): operator update =
 * Overlap::update (src/both_3d/overlap.h:207-216: links, lambda bounds by
 * power iterations, Zolotarev coefficients) when lmin = lmax = 0, or fixed
 * bounds lmin < lmax; phi = D_ov^dag xi; eta = (D_ov^dag D_ov)^{-1} phi by
 * the outer CG to tol (pole solves to tol_inner); force = qed3_overlap_force.
 * ov's Wilson operator must live on lat. */
int qed3_hmc_overlap(qed3_lattice* lat, qed3_overlap* ov, qed3_rng* rng, double* A, double beta, int compact,
                     int exact, double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double lmin,
                     double lmax, double tol, double tol_inner, int no_reject, int* accepted, double* dH,
                     int* cg_iters, void* stream);
int qed3_hmc_pure_gauge(qed3_lattice* lat, qed3_rng* rng, double* A, double beta, int compact, int exact,
                        double tmax, int nsteps, int no_reject, int* accepted, double* dH, void* stream);
/* One S^2 x S^1 HMC trajectory on the device links A (in place): HMC2::run
 * with the anisotropic gauge action (at, gsq) and npf Wilson pseudofermions
 * of the S^2 x S^1 operator e, QED3_INTEGRATOR_LEAPFROG_ML or _LEAPFROG; rng must hold
 * Nt n_links link engines and Nt n_sites site engines (ParallelRngExt's
 * layout: spatial momenta from the link engines, temporal momenta and the
 * pseudofermion sources from the site engines); solves to tol, precision
 * QED3_PREC_F64 (the reference's recurrence) or QED3_PREC_F32 (FP32 iterations
 * with FP64 reliable updates, same certificate). */
int qed3_hmc_ext(qed3_dirac_ext* e, qed3_rng* rng, double* A, double at, double gsq, double tmax, int nsteps,
                 int nsteps_inner, int npf, int integrator, double tol, int precision, int no_reject, int* accepted,
                 double* dH, int* cg_iters, void* stream);
/* HMC2::run with Overlap<DiracExt> pseudofermions (the reference's IS_OVERLAP
 * hmc.cu on S^2 x S^1): as qed3_hmc_ext with phi = D_ov^dag xi, eta by the
 * outer CG on D_ov^dag D_ov (tol; poles to tol_inner), the overlap force, and
 * the bounds fixed (lambda_min, lambda_max > 0) or recomputed by Lanczos at
 * every link update (both 0). */
int qed3_hmc_ext_overlap(qed3_overlap_ext* ov, qed3_rng* rng, double* A, double at, double gsq, double tmax,
                         int nsteps, int nsteps_inner, int npf, int integrator, double tol, double tol_inner,
                         double lambda_min, double lambda_max, int no_reject, int* accepted, double* dH,
                         int* cg_iters, void* stream);

/* ======================================================================
 * Overlap operator  --  replaces Overlap<WilsonDirac> (src/both_3d/overlap.h:137-390):
 * D_ov = 1 + X r(X^dag X), X = D_W / lambda_max, r = Zolotarev approximation of
 * (.)^{-1/2} of order zolo_order (n/2 poles).  All poles are solved by ONE
 * FP64 multi-shift CG (one Krylov space; poles that stall just above the
 * tolerance get a mixed-precision defect correction), FP64 true residuals.
 * ====================================================================== */
int qed3_overlap_create(qed3_dirac* dw, int zolo_order, int precision, qed3_overlap** out);
int qed3_overlap_destroy(qed3_overlap* ov);
/* Overlap::update -> compute_lambda_max + Zolotarev::update (:207-306).  Pass
 * lambda_min, lambda_max > 0 to set the spectral bounds of D_W directly, or
 * <= 0 to estimate them with the reference's power / inverse power iterations
 * (inner CG tolerance tol_outer). */
int qed3_overlap_update(qed3_overlap* ov, double lambda_min, double lambda_max, double tol_outer, void* stream);
/* npoles_fp64: leading (smallest-shift) poles whose condition number is too
 * large for mixed-precision inner iterations (they would need FP64 in the
 * batched alternative to the multi-shift solve; 0 when the overlap was
 * created with QED3_PREC_F64). */
int qed3_overlap_info(const qed3_overlap* ov, double* lambda_min, double* lambda_max, double* k, double* delta,
                      int* npoles, int* npoles_fp64);
/* mult / adj / DHD / DDH_deviceAsyncLaunch (:309-390): op = QED3_OP_D (D_ov),
 * QED3_OP_DDAG (D_ov^dag), QED3_OP_DDAGD or QED3_OP_DDDAG (D_ov + D_ov^dag,
 * which equals D_ov^dag D_ov for the exact overlap).  tol_inner: pole solves'
 * relative residual.  report: the worst pole (iterations, true residual); a
 * pole that stalls within 100 x tol_inner sets report->status but does not fail
 * the call (ill-conditioned poles reach the FP64 floor there). */
int qed3_overlap_apply(qed3_overlap* ov, int op, double* out, const double* in, double tol_inner,
                       qed3_solve_report* report, void* stream);

/* Overlap pseudofermion force for all links at once -- replaces
 * Overlap::precalc_grad_deviceAsyncLaunch + grad_deviceAsyncLaunch
 * (src/both_3d/overlap.h:393-470, one sparse product and dot per pole and
 * link): F[l] = -2 d/dA_l Re<eta, D_ov eta>.  eta: device complex128,
 * reference order; F: device [n_links].  report: the worse of the two
 * multi-shift pole solves. */
int qed3_overlap_force(qed3_overlap* ov, const double* eta, double* F, double tol_inner, qed3_solve_report* report,
                       void* stream);
/* Outer CG on D_ov^dag D_ov (Overlap::DHD) x = b, as MatPoly::solve over the
 * DHD wrapper (src/both_3d/prop_nontriv.cu:242-260); device complex128 x, b.
 * report: outer iterations, true_rel_res = ||b - D_ov^dag D_ov x||/||b||
 * recomputed after convergence, reliable_updates = the largest inner pole
 * iteration count. */
int qed3_overlap_solve(qed3_overlap* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                       qed3_solve_report* report, void* stream);
/* The same outer solve with options (no counterpart in the reference, whose
 * outer CG is qed3_overlap_solve): QED3_OVSOLVE_CHIRAL solves the two
 * chirality sectors one after the other -- D_ov + D_ov^dag commutes with
 * gamma5 and is 2 P_c D_ov P_c on sector c, so each iteration needs one pole
 * solve instead of two.  Every solve is certified by
 * ||b - (D_ov + D_ov^dag) x|| / ||b|| recomputed with certified pole solves to
 * tol_inner, and restarted on that residual when it is above tol. */
#define QED3_OVSOLVE_CHIRAL 1
int qed3_overlap_solve2(qed3_overlap* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                        int flags, qed3_solve_report* report, void* stream);
/* Low-mode projection of the sign function (no counterpart in the reference,
 * whose Overlap approximates sign(H) on the whole spectrum,
 * src/both_3d/overlap.h:207-306): the nev eigenvectors h_i of
 * H = gamma5 D_W / lambda_max nearest zero (Lanczos on D_W^dag D_W with full
 * reorthogonalisation to residual tol x its largest eigenvalue, at most
 * maxsteps steps, then Rayleigh-Ritz with H) are treated exactly,
 * sign(H) = sum_i sign(mu_i) h_i h_i^dag + H r(H^2)(1 - P), and the
 * Zolotarev range starts at the (nev+1)-th |mu| (times 1 - margin).  That
 * removes the near-zero modes of H_W at M5 < 0 from every pole solve.  Needs
 * qed3_overlap_update first (it keeps lambda_max); nev = 0 switches the
 * projection off; a later qed3_overlap_update drops it.  While it is on,
 * qed3_overlap_force refuses (the force is for the unprojected sign
 * function). */
int qed3_overlap_project_low_modes(qed3_overlap* ov, int nev, double tol, int maxsteps, double margin, void* stream);
/* How the poles are solved (no counterpart in the reference, which runs one
 * CG per pole on its own stream): QED3_POLES_MULTISHIFT (default) -- one FP64
 * multi-shift CG for all poles, one stencil pass per iteration;
 * QED3_POLES_BATCHED -- every pole its own mixed-precision CG (FP32
 * iterations on FP32 or BF16-halo vectors, FP64 reliable updates and FP64
 * true-residual certificates) in one persistent batched launch, the
 * right-hand side broadcast; poles too ill-conditioned for FP32 inner
 * iterations (condition above 2e5) run in FP64 in a second launch. */
/* Massive overlap D(m) = (1 - m/2) D_ov + m, m in [0, 2) (no counterpart in
 * the reference, whose Overlap is massless): qed3_overlap_apply returns
 * D(m), D(m)^dag and D(m)^dag D(m) = (1 - m^2/4)(D_ov + D_ov^dag) + m^2, and
 * the outer solves invert the latter.  The massless D_ov^dag D_ov is
 * singular on configurations with topological charge (|Q| exact zero modes)
 * and has near-zero modes at strong coupling; the mass bounds its spectrum
 * below by m^2.  qed3_overlap_force refuses a nonzero mass. */
int qed3_overlap_set_mass(qed3_overlap* ov, double mass);
#define QED3_POLES_MULTISHIFT 0
#define QED3_POLES_BATCHED 1
int qed3_overlap_set_pole_solver(qed3_overlap* ov, int mode);
/* nev in use, max ||H h_i - mu_i h_i||, Lanczos steps, mu[nev] (host, may be NULL) */
int qed3_overlap_low_modes_info(const qed3_overlap* ov, int* nev, double* max_residual, int* lanczos_steps,
                                double* mu);

/* Multi-shift CG: x[m] = (D^dag D + shifts[m])^{-1} b for m < nshifts (<= 64),
 * all shifts in one Krylov space (one D^dag D per iteration for all shifts),
 * FP64 -- replaces the per-pole MatPoly::solve calls of Overlap
 * (src/both_3d/overlap.h:309-358).  shifts: host, >= 0; x: device complex128,
 * nshifts vectors back to back; b: device complex128 (reference order).
 * reports[m] (host, may be NULL): iterations at which shift m stopped, its
 * FP64 true residual ||b - (D^dag D + shift) x|| / ||b||, status; ms: device time. */
int qed3_multishift_solve(qed3_dirac* d, int nshifts, const double* shifts, double* x, const double* b, double tol,
                          int maxiter, qed3_solve_report* reports, float* ms, void* stream);

/* ======================================================================
 * Zolotarev coefficients  --  replaces Zolotarev(k, n) / Zolotarev::update
 * (src/both_3d/overlap.h:7-116): r(x) = C x (1 + sum_m A[m]/(x^2 - k^2/cp[m])).
 * Host arrays of length n/2+1 (index 0 unused); scal = {M, lambda_inv, E, C}.
 * Returns the size n/2+1 through *size.
 * ====================================================================== */
int qed3_zolotarev(double k, int n, double* c, double* cp, double* A, double* scal, int* size);

/* ======================================================================
 * Learned preconditioner and preconditioned CG  --  no counterpart in the
 * reference (its solvers are unpreconditioned CG: src/both_3d/cg_cuda.h,
 * sparse_matrix.h).  N(r) = a^2 r + G^dag G r, G = L_layers o ... o L_1,
 * each layer a gauge-covariant parallel-transport convolution over complex
 * channels, L(h)[c] = sum_c' W0[c,c'] h[c'] + W1[c,c'] Hd h[c'] + W2[c,c'] Ho h[c'],
 * where Hd / Ho are the spin-diagonal / off-diagonal parts of the Dirac hop
 * restricted to the solver's per-SM site blocks.  N is hermitian positive
 * definite by construction.  Trained on the GPU (hand-written forward,
 * backward and Adam kernels) on residual / error pairs taken from the
 * solver's own iterates, loss 1 - |<z,r>|^2 / (<z,A z> <e,r>) with A = D^dag D.
 * ====================================================================== */
/* channels in [1, 64], layers in [1, 3] (the solver takes 1 or 2); the block partition is the one of the
 * register-resident solvers on the current device. */
int qed3_lpc_create(qed3_dirac* d, int channels, int layers, unsigned seed, qed3_lpc** out);
int qed3_lpc_destroy(qed3_lpc* pc);
/* nparams: complex parameters (layer l: 3 x Cout x Cin, row-major [j][c][c'],
 * then a as (a, 0)); block_sites: sites per block; npairs: training pairs held. */
int qed3_lpc_info(const qed3_lpc* pc, int* nparams, int* block_sites, int* npairs);
/* host arrays of 2*nparams doubles (re, im interleaved); set resets Adam. */
int qed3_lpc_get_weights(const qed3_lpc* pc, double* w);
int qed3_lpc_set_weights(qed3_lpc* pc, const double* w);
/* z = N r with the hop blocks of the operator pc was created on.  r, z: device
 * complex128, nrhs vectors of 2*n_sites back to back, reference order.
 * form 0: layer-by-layer (the training network); form 1: the collapsed word
 * form the solver applies (identical up to rounding). */
int qed3_lpc_apply(qed3_lpc* pc, int form, double* z, const double* r, int nrhs, void* stream);
/* loss and its gradient (host grad[2*nparams]) on pairs (r, e) of the creating
 * operator; device complex128 inputs as in qed3_lpc_apply. */
int qed3_lpc_loss_grad(qed3_lpc* pc, const double* r, const double* e, int nrhs, double* loss, double* grad,
                       void* stream);
/* Adds nsrc * nsnap training pairs from operator d (same lattice): Gaussian
 * sources (seeded), x* from a full solve, x_k = CG stopped after snapshots[k]
 * iterations (0: x_k = 0), pair (b - A x_k, x* - x_k) / |b - A x_k|. */
int qed3_lpc_collect(qed3_lpc* pc, qed3_dirac* d, int nsrc, unsigned seed, const int* snapshots, int nsnap,
                     int precision);
/* steps of Adam (learning rate lr), each on `batch` pairs of one operator drawn
 * at random; loss_history: host [steps] or NULL. */
int qed3_lpc_train(qed3_lpc* pc, int steps, int batch, double lr, unsigned seed, double* loss_history);
/* Channel mixing of the 16 -> 16 layers on the tensor cores (tcgen05, BF16
 * operands, FP32 accumulation; default on for 16 channels and 2 layers) or in
 * FP32 on the CUDA cores (enable = 0).  QED3_ERR_ARG if the network has no
 * 16 -> 16 layer. */
int qed3_lpc_set_tensor_cores(qed3_lpc* pc, int enable);
/* Preconditioned CG on D^dag D + shift with N applied block-locally inside the
 * persistent kernel.  Same arguments, certificate and report as qed3_cg_solve;
 * precision QED3_PREC_F32 or QED3_PREC_BF16 (halo copies), FP64 reliable
 * updates and true residual.  d: any operator on pc's lattice. */
int qed3_pcg_solve(qed3_dirac* d, qed3_lpc* pc, double* x, const double* b, const qed3_solve_params* params,
                   qed3_solve_report* report, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QED3_GB300_H */
