// Overlap operator D_ov = 1 + X r(X^dag X), X = D_W / lambda_max, r the
// Zolotarev approximation of (.)^{-1/2} (the sign function of gamma5 X).
//
// Replaces Overlap (src/both_3d/overlap.h:137-390).  The reference solves one
// CG per pole on OpenMP threads and CUDA streams (:309-332); here the npoles
// systems (D^dag D + lambda_max^2 sigma_m) z_m = xi, sigma_m = -k^2/cp_m > 0,
// are ONE FP64 multi-shift CG (mshift.cu: one Krylov space, one stencil pass
// per iteration for all poles) with an FP64 true-residual certificate per
// pole; the alternative, one batched persistent launch of shifted mixed-
// precision CGs with the right-hand side broadcast (batched.cu), is kept for
// comparison.  Then
//   D_ov xi     = xi + (C/lambda_max) D (xi + sum_m A_m lambda_max^2 z_m)
//   D_ov^dag xi = xi + C (y0 + sum_m A_m lambda_max^2 y_m),  y0 = D^dag xi / lambda_max
// lambda_min/max come from the reference's procedure (power iteration on
// D^dag D with its geometric extrapolation, inverse power iteration with CG,
// :217-306) or are passed in.

#include <cmath>
#include <vector>

#include "batched_impl.h"
#include "blas_impl.h"
#include "dirac_impl.h"
#include "gauge_impl.h"
#include "mshift_impl.h"
#include "handles.h"
#include "overlap_impl.h"
#include "qed3_internal.h"

struct qed3_overlap_s {
  qed3_dirac_s* d = nullptr;
  int order = 21, prec = QED3_PREC_F32;
  qed3::ZoloCoeffs z;
  double lmin = 0, lmax = 0;
  bool ready = false;
  qed3_batch_s* batch = nullptr;     // poles nh..np-1 in the overlap's precision
  qed3_batch_s* batch_hi = nullptr;  // poles 0..nh-1 (ill-conditioned) in FP64
  int nh = 0, nlo = 0;               // current split
  bool multishift = true;            // all poles through the FP64 multi-shift CG (false: batched launches)
  double* Z = nullptr;     // [npoles][2 Ns] complex
  double* y = nullptr;     // [2 Ns] complex
  double* w = nullptr;
  double* y0 = nullptr;
  double* q = nullptr;
  double* part = nullptr;  // reduction scratch
  // force: second pole set and internal-order copies; outer solve: CG vectors
  double* Yp = nullptr;    // [npoles][2 Ns] complex
  double* fi = nullptr;    // [4 npoles + 2][Ns] internal-order two-spinors (4 doubles per site)
  double *sr = nullptr, *sp = nullptr, *sq = nullptr;
  // multi-shift scratch (internal-order FP64 fields, [npoles][Ns] each)
  qed3::S64* msX = nullptr;
  qed3::S64* msP = nullptr;
};

namespace qed3 {

static int ov_alloc(qed3_overlap_s* ov) {
  const size_t n = size_t(4) * ov->d->Ns;  // doubles per vector
  const int np = ov->order / 2;
  QED3_CUDA_TRY(cudaMalloc(&ov->Z, n * np * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ov->y, n * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ov->w, n * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ov->y0, n * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ov->q, n * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ov->part, 2048 * sizeof(double)));
  qed3_dirac_s* ops[1] = {ov->d};
  const int nr[1] = {np};
  ov->nh = 0;
  ov->nlo = np;
  return batch_create(1, ops, nr, ov->prec, 0, 0, &ov->batch);
}

// Condition number above which a pole system leaves the mixed-precision
// launch: its inner FP32 (BF16-halo) iterations stagnate before the tolerance
// (measured at n=32, beta=1.4, M5=-1: lambda_min/lambda_max = 1.5e-4 gives
// kappa = 4e7 for the smallest shift, where FP32-inner CG stalls near 1e-9).
static double mixed_cond_limit(int prec) { return prec == QED3_PREC_BF16 ? 2e4 : 2e5; }

// Splits the poles between the two batched launches: pole m's system
// D^dag D + lmax^2 s_m has condition (1 + s_m) / (k^2 + s_m); the leading
// (smallest-shift) poles above the limit run in FP64.
static int ov_split(qed3_overlap_s* ov) {
  const int np = ov->order / 2;
  int nh = 0;
  if (ov->prec != QED3_PREC_F64) {
    const double k2 = ov->z.k * ov->z.k;
    for (int m = 1; m <= np; m++) {
      const double s = -k2 / ov->z.cp[m];
      if ((1.0 + s) / (k2 + s) > mixed_cond_limit(ov->prec)) nh = m;  // prefix up to the last hard pole
    }
  }
  if (nh == ov->nh && ov->nlo == np - nh) return QED3_OK;
  if (ov->batch) batch_destroy(ov->batch);
  if (ov->batch_hi) batch_destroy(ov->batch_hi);
  ov->batch = ov->batch_hi = nullptr;
  qed3_dirac_s* ops[1] = {ov->d};
  int rc;
  if (np - nh > 0) {
    const int nr[1] = {np - nh};
    if ((rc = batch_create(1, ops, nr, ov->prec, 0, 0, &ov->batch))) return rc;
  }
  if (nh > 0) {
    const int nr[1] = {nh};
    if ((rc = batch_create(1, ops, nr, QED3_PREC_F64, 0, 0, &ov->batch_hi))) return rc;
  }
  ov->nh = nh;
  ov->nlo = np - nh;
  return QED3_OK;
}

void overlap_destroy(qed3_overlap_s* ov) {
  if (!ov) return;
  if (ov->batch) batch_destroy(ov->batch);
  if (ov->batch_hi) batch_destroy(ov->batch_hi);
  void* p[] = {ov->Z, ov->y, ov->w, ov->y0, ov->q, ov->part, ov->Yp, ov->fi, ov->sr, ov->sp, ov->sq, ov->msX, ov->msP};
  for (void* x : p)
    if (x) cudaFree(x);
  delete ov;
}

int overlap_create(qed3_dirac_s* d, int order, int prec, qed3_overlap_s** out) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  if (order < 3 || order / 2 > kMaxPoles) return fail(QED3_ERR_ARG, "Zolotarev order must be in [3, 129]");
  auto* ov = new qed3_overlap_s;
  ov->d = d;
  ov->order = order;
  ov->prec = prec;
  const int rc = ov_alloc(ov);
  if (rc) {
    overlap_destroy(ov);
    return rc;
  }
  *out = ov;
  return QED3_OK;
}

// Power iteration of the reference (src/both_3d/overlap.h:226-262): returns the
// extrapolated dominant eigenvalue of D^dag D (inverse = false) or of its inverse.
static int power_iteration(qed3_overlap_s* ov, bool inverse, double TOL, int MAXITER, double tol_outer, double* lam,
                           cudaStream_t st) {
  qed3_dirac_s* d = ov->d;
  const long long nc = 2LL * d->Ns, nd = 2 * nc;
  std::vector<double> q0(size_t(nd), 0.0);
  q0[0] = std::sqrt(0.5);  // q[0] = q[1] = 1/sqrt(2) as complex entries (re parts)
  q0[2] = std::sqrt(0.5);
  QED3_CUDA_TRY(cudaMemcpyAsync(ov->q, q0.data(), nd * sizeof(double), cudaMemcpyHostToDevice, st));
  double mu_0 = 1.0, mu_m1 = 1.0, mu_m2 = 1.0, lambda = 100.0, lambda_old = 1000.0;
  qed3_solve_params p{tol_outer, 0, QED3_PREC_F32, 0.1, 0.0, 0};
  int rc;
  for (int i = 0; i < MAXITER; i++) {
    if (!inverse) rc = dirac_apply_ref(d, QED3_OP_DDAGD, ov->w, ov->q, st);
    else rc = cg_solve(d, ov->w, ov->q, &p, nullptr, st);
    if (rc) return rc;
    double nrm, dr;
    if ((rc = vec_zdot(nc, ov->w, ov->w, ov->part, &nrm, nullptr, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0 / std::sqrt(nrm), ov->w, 0.0, ov->w, ov->q, st))) return rc;
    if ((rc = vec_zdot(nc, ov->w, ov->q, ov->part, &dr, nullptr, st))) return rc;
    mu_m2 = mu_m1;
    mu_m1 = mu_0;
    mu_0 = dr;
    const double r = (mu_0 - mu_m1) / (mu_m1 - mu_m2);
    const double a = (mu_0 - mu_m1) / std::pow(r, i - 1) / (r - 1);
    lambda_old = lambda;
    lambda = mu_0 - a * std::pow(r, i);
    if (std::abs(lambda_old - lambda) / std::abs(lambda) < TOL) break;
  }
  *lam = lambda;
  return QED3_OK;
}

int overlap_update(qed3_overlap_s* ov, double lmin, double lmax, double tol_outer, cudaStream_t st) {
  if (!(lmin > 0 && lmax > 0)) {
    const double TOL = 1e-8;
    double lam = 0, lam2 = 0;
    int rc = power_iteration(ov, false, TOL, 500, tol_outer, &lam, st);
    if (rc) return rc;
    if ((rc = power_iteration(ov, true, TOL, 500, tol_outer, &lam2, st))) return rc;
    lmin = std::sqrt((1.0 - 100 * TOL) / lam2);
    lmax = std::sqrt((1.0 + 100 * TOL) * lam);
  }
  if (!(lmin < lmax)) return fail(QED3_ERR_ARG, "need 0 < lambda_min < lambda_max");
  ov->lmin = lmin;
  ov->lmax = lmax;
  int rc = zolotarev_coeffs(lmin / lmax, ov->order, ov->z);
  if (rc) return rc;
  if ((rc = ov_split(ov))) return rc;
  ov->ready = true;
  return QED3_OK;
}

// All poles with one right-hand side: out_m = (D^dag D + lmax^2 sigma_m)^{-1} rhs,
// through one FP64 multi-shift CG (one Krylov space, one D^dag D per iteration
// for all poles; mshift.cu).  It beats the batched launches (every pole its
// own mixed-precision system, the right-hand side broadcast; kept for
// comparison) also when every pole is well conditioned: n=16, M5=-1, 20
// poles, k = 0.0058: 47 ms against 104 ms, since the slowest pole sets the
// iteration count of both and the multi-shift iteration does one stencil
// pass instead of twenty.
static int pole_solves(qed3_overlap_s* ov, const double* rhs, double* out, double tol, qed3_solve_report* worst,
                       cudaStream_t st) {
  const int np = ov->order / 2;
  const long long nd = 4LL * ov->d->Ns;
  std::vector<double> shifts(np);
  for (int m = 1; m <= np; m++) shifts[m - 1] = ov->lmax * ov->lmax * (-ov->z.k * ov->z.k / ov->z.cp[m]);
  std::vector<qed3_solve_report> reps(np);
  qed3_solve_report w{};
  const double* bs[1] = {rhs};
  if (ov->multishift) {
    if (!ov->msX) {
      QED3_CUDA_TRY(cudaMalloc(&ov->msX, size_t(np) * nd * sizeof(double)));
      QED3_CUDA_TRY(cudaMalloc(&ov->msP, size_t(np) * nd * sizeof(double)));
    }
    float ms = 0;
    const int rc = mshift_solve(ov->d, np, shifts.data(), rhs, out, ov->msX, ov->msP, tol, 200000, reps.data(), &ms, st);
    if (rc) return rc;
    w.ms = ms;
  }
  for (int part = 0; part < 2 && !ov->multishift; part++) {
    const bool hi = part == 0;
    const int m0 = hi ? 0 : ov->nh, cnt = hi ? ov->nh : ov->nlo;
    if (cnt == 0) continue;
    double* xs[1] = {out + size_t(m0) * nd};
    const double* sh[1] = {shifts.data() + m0};
    qed3_solve_params p{tol, 0, hi ? QED3_PREC_F64 : ov->prec, 0.1, 0.0, QED3_SOLVE_BCAST_B};
    float ms = 0;
    const int rc = batch_solve(hi ? ov->batch_hi : ov->batch, xs, bs, sh, &p, reps.data() + m0, &ms, st);
    if (rc) return rc;
    w.ms += ms;
  }
  for (auto& r : reps) {
    if (r.status != QED3_OK) w.status = r.status;
    w.iters = std::max(w.iters, r.iters);
    w.reliable_updates = std::max(w.reliable_updates, r.reliable_updates);
    w.true_rel_res = std::max(w.true_rel_res, r.true_rel_res);
  }
  if (worst) *worst = w;
  // A pole that ends within 100 x tol (the FP64 floor of an ill-conditioned
  // pole with a low-mode right-hand side) does not abort the product: its
  // status and true residual are in the report, and an outer solve judges the
  // result by its own certificate.
  if (w.status == QED3_OK || w.true_rel_res <= 100.0 * tol) return QED3_OK;
  return fail(w.status, "a pole solve did not converge");
}

int overlap_apply(qed3_overlap_s* ov, int op, double* out, const double* in, double tol, qed3_solve_report* rep,
                  cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_update first");
  qed3_dirac_s* d = ov->d;
  const long long nd = 4LL * d->Ns;
  const int np = ov->order / 2;
  const double l2 = ov->lmax * ov->lmax;
  std::vector<double> coef(np);
  for (int m = 1; m <= np; m++) coef[m - 1] = ov->z.A[m] * l2;
  const double C = ov->z.C;
  int rc;
  qed3_solve_report r1{}, r2{};
  const bool mult = (op == QED3_OP_D || op == QED3_OP_DDAGD || op == QED3_OP_DDDAG);
  const bool adj = (op == QED3_OP_DDAG || op == QED3_OP_DDAGD || op == QED3_OP_DDDAG);
  if (mult) {
    if ((rc = pole_solves(ov, in, ov->Z, tol, &r1, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), ov->Z, in, ov->y, st))) return rc;  // y = xi + sum A l2 z
    if ((rc = dirac_apply_ref(d, QED3_OP_D, ov->w, ov->y, st))) return rc;          // w = D y
  }
  if (adj) {
    if ((rc = dirac_apply_ref(d, QED3_OP_DDAG, ov->y0, in, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0 / ov->lmax, ov->y0, 0.0, ov->y0, ov->y0, st))) return rc;  // y0 = D^dag xi / lmax
    if ((rc = pole_solves(ov, ov->y0, ov->Z, tol, &r2, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), ov->Z, ov->y0, ov->y, st))) return rc;  // y = y0 + sum A l2 y_m
  }
  if (mult && adj) {
    // out = 2 xi + (C/lmax) w + C y
    if ((rc = vec_axpby(nd, C / ov->lmax, ov->w, C, ov->y, ov->q, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0, ov->q, 2.0, in, out, st))) return rc;
  } else if (mult) {
    if ((rc = vec_axpby(nd, C / ov->lmax, ov->w, 1.0, in, out, st))) return rc;
  } else {
    if ((rc = vec_axpby(nd, C, ov->y, 1.0, in, out, st))) return rc;
  }
  if (rep) {
    qed3_solve_report w = mult ? r1 : r2;
    if (mult && adj) {
      w.iters = std::max(r1.iters, r2.iters);
      w.true_rel_res = std::max(r1.true_rel_res, r2.true_rel_res);
      w.ms = r1.ms + r2.ms;
    }
    *rep = w;
  }
  return QED3_OK;
}

// Overlap pseudofermion force for all links at once (Overlap::precalc_grad +
// grad_deviceAsyncLaunch, src/both_3d/overlap.h:393-470, which loops over
// links with one sparse product and dot per pole and link):
//   F_l = -2C/lmax [ sum_m A_m (-Re<X Z_m, dD Y_m> - Re<X Y_m, dD Z_m>) + Re<eta, dD w> ],
//   Z_m = (X^dag X + s_m)^{-1} eta, Y_m = (X^dag X + s_m)^{-1} X^dag eta, w = eta + sum_m A_m Z_m.
// With the pole solves' Z'_m = Z_m / lmax^2 (the batched systems are D^dag D + lmax^2 s_m):
//   F_l = sum_m 2 C A_m lmax^2 (Re<D Z'_m, dD Y'_m> + Re<D Y'_m, dD Z'_m>) - 2C/lmax Re<eta, dD w>.
int overlap_force(qed3_overlap_s* ov, const double* eta, double* F, double tol, qed3_solve_report* rep,
                  cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_update first");
  qed3_dirac_s* d = ov->d;
  const int Ns = d->Ns;
  const long long nd = 4LL * Ns;
  const int np = ov->order / 2;
  if (!ov->Yp) QED3_CUDA_TRY(cudaMalloc(&ov->Yp, size_t(nd) * np * sizeof(double)));
  if (!ov->fi) QED3_CUDA_TRY(cudaMalloc(&ov->fi, size_t(4 * np + 2) * Ns * 4 * sizeof(double)));
  const double l2 = ov->lmax * ov->lmax;
  int rc;
  qed3_solve_report r1{}, r2{};
  if ((rc = dirac_apply_ref(d, QED3_OP_DDAG, ov->y0, eta, st))) return rc;
  if ((rc = vec_axpby(nd, 1.0 / ov->lmax, ov->y0, 0.0, ov->y0, ov->y0, st))) return rc;
  if ((rc = pole_solves(ov, eta, ov->Z, tol, &r1, st))) return rc;
  if ((rc = pole_solves(ov, ov->y0, ov->Yp, tol, &r2, st))) return rc;
  std::vector<double> coef(np), c(np);
  for (int m = 1; m <= np; m++) {
    coef[m - 1] = ov->z.A[m] * l2;
    c[m - 1] = 2.0 * ov->z.C * ov->z.A[m] * l2;
  }
  if ((rc = vec_pole_sum(nd, np, coef.data(), ov->Z, eta, ov->w, st))) return rc;  // w = eta + sum A l2 Z'
  const size_t vs = size_t(Ns) * 4;  // doubles per internal two-spinor field
  auto fld = [&](size_t k) { return reinterpret_cast<S64*>(ov->fi + k * vs); };
  S64* ZI = fld(0);
  S64* YI = fld(np);
  S64* DZ = fld(2 * size_t(np));
  S64* DY = fld(3 * size_t(np));
  S64* EI = fld(4 * size_t(np));
  S64* WI = fld(4 * size_t(np) + 1);
  if ((rc = field_import(d, QED3_PREC_F64, ZI, ov->Z, np, st))) return rc;
  if ((rc = field_import(d, QED3_PREC_F64, YI, ov->Yp, np, st))) return rc;
  if ((rc = field_import(d, QED3_PREC_F64, EI, eta, 1, st))) return rc;
  if ((rc = field_import(d, QED3_PREC_F64, WI, ov->w, 1, st))) return rc;
  if ((rc = dirac_apply_field(d, QED3_OP_D, QED3_PREC_F64, DZ, ZI, np, st))) return rc;
  if ((rc = dirac_apply_field(d, QED3_OP_D, QED3_PREC_F64, DY, YI, np, st))) return rc;
  if ((rc = overlap_force_links(d, np, c.data(), -2.0 * ov->z.C / ov->lmax, ZI, YI, DZ, DY, EI, WI, F, st)))
    return rc;
  if (rep) {
    qed3_solve_report w = r1;
    w.iters = std::max(r1.iters, r2.iters);
    w.true_rel_res = std::max(r1.true_rel_res, r2.true_rel_res);
    w.ms = r1.ms + r2.ms;
    *rep = w;
  }
  return QED3_OK;
}

// Outer CG on D_ov^dag D_ov (= D_ov + D_ov^dag for the overlap; Overlap::DHD,
// src/both_3d/overlap.h:363-375) as the reference's MatPoly::solve over a
// LinOpWrapper of DHD (src/both_3d/prop_nontriv.cu:242-260); every product is
// one pair of batched pole launches.  The report's true_rel_res is
// ||b - D_ov^dag D_ov x|| / ||b|| recomputed after convergence.
int overlap_solve(qed3_overlap_s* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                  qed3_solve_report* rep, cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_update first");
  const long long nd = 4LL * ov->d->Ns, nc = nd / 2;
  if (!ov->sr) {
    QED3_CUDA_TRY(cudaMalloc(&ov->sr, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->sp, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->sq, nd * sizeof(double)));
  }
  cudaEvent_t e0, e1;
  QED3_CUDA_TRY(cudaEventCreate(&e0));
  QED3_CUDA_TRY(cudaEventCreate(&e1));
  QED3_CUDA_TRY(cudaEventRecord(e0, st));
  int rc;
  double bb = 0;
  if ((rc = vec_zdot(nc, b, b, ov->part, &bb, nullptr, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(x, 0, nd * sizeof(double), st));
  QED3_CUDA_TRY(cudaMemcpyAsync(ov->sr, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(ov->sp, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double rr = bb;
  int it = 0, status = QED3_ERR_NOCONV, inner_max = 0;
  if (bb == 0.0) status = QED3_OK;
  while (status != QED3_OK && it < maxiter) {
    qed3_solve_report ir{};
    if ((rc = overlap_apply(ov, QED3_OP_DDAGD, ov->sq, ov->sp, tol_inner, &ir, st))) return rc;
    inner_max = std::max(inner_max, ir.iters);
    double pq = 0;
    if ((rc = vec_zdot(nc, ov->sp, ov->sq, ov->part, &pq, nullptr, st))) return rc;
    const double al = rr / pq;
    if ((rc = vec_axpby(nd, al, ov->sp, 1.0, x, x, st))) return rc;
    if ((rc = vec_axpby(nd, -al, ov->sq, 1.0, ov->sr, ov->sr, st))) return rc;
    double rn = 0;
    if ((rc = vec_zdot(nc, ov->sr, ov->sr, ov->part, &rn, nullptr, st))) return rc;
    it++;
    if (!(std::isfinite(rn) && std::isfinite(al))) break;
    if (rn < tol * tol * bb) {
      status = QED3_OK;
      break;
    }
    if ((rc = vec_axpby(nd, 1.0, ov->sr, rn / rr, ov->sp, ov->sp, st))) return rc;
    rr = rn;
  }
  // certificate: r = b - A x with the same operator
  double tr = 0;
  if (bb > 0) {
    if ((rc = overlap_apply(ov, QED3_OP_DDAGD, ov->sq, x, tol_inner, nullptr, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0, b, -1.0, ov->sq, ov->sq, st))) return rc;
    if ((rc = vec_zdot(nc, ov->sq, ov->sq, ov->part, &tr, nullptr, st))) return rc;
  }
  QED3_CUDA_TRY(cudaEventRecord(e1, st));
  QED3_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rep) {
    rep->status = status;
    rep->iters = it;
    rep->reliable_updates = inner_max;  // the largest inner (pole) iteration count of any product
    rep->true_rel_res = bb > 0 ? std::sqrt(tr / bb) : 0.0;
    rep->ms = ms;
  }
  return QED3_OK;
}

}  // namespace qed3

namespace qed3 {
qed3_dirac_s* overlap_dirac(qed3_overlap_s* ov) { return ov->d; }

int overlap_info(const qed3_overlap_s* ov, double* lmin, double* lmax, double* k, double* delta, int* np,
                 int* np_fp64) {
  if (np_fp64) *np_fp64 = ov->nh;
  if (lmin) *lmin = ov->lmin;
  if (lmax) *lmax = ov->lmax;
  if (k) *k = ov->ready ? ov->z.k : 0.0;
  if (delta) *delta = ov->ready ? (ov->z.lambda_inv - 1.0) / (ov->z.lambda_inv + 1.0) : 0.0;
  if (np) *np = ov->order / 2;
  return QED3_OK;
}
}  // namespace qed3
