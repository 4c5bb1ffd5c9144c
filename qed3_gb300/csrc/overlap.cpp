// Overlap operator D_ov = 1 + X r(X^dag X), X = D_W / lambda_max, r the
// Zolotarev approximation of (.)^{-1/2} (the sign function of gamma5 X).
//
// Replaces Overlap (src/both_3d/overlap.h:137-390).  The reference solves one
// CG per pole on OpenMP threads and CUDA streams (:309-332); here all poles
// are ONE batched persistent launch of shifted CGs (batched.cu) that share
// every stencil read: the right-hand side is broadcast to the npoles systems
// (D^dag D + lambda_max^2 sigma_m) z_m = xi, sigma_m = -k^2/cp_m > 0, in
// mixed precision with FP64 reliable updates and an FP64 true-residual
// certificate per pole.  Then
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
#include "handles.h"
#include "overlap_impl.h"
#include "qed3_internal.h"

struct qed3_overlap_s {
  qed3_dirac_s* d = nullptr;
  int order = 21, prec = QED3_PREC_F32;
  qed3::ZoloCoeffs z;
  double lmin = 0, lmax = 0;
  bool ready = false;
  qed3_batch_s* batch = nullptr;
  double* Z = nullptr;     // [npoles][2 Ns] complex
  double* y = nullptr;     // [2 Ns] complex
  double* w = nullptr;
  double* y0 = nullptr;
  double* q = nullptr;
  double* part = nullptr;  // reduction scratch
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
  return batch_create(1, ops, nr, ov->prec, 0, 0, &ov->batch);
}

void overlap_destroy(qed3_overlap_s* ov) {
  if (!ov) return;
  if (ov->batch) batch_destroy(ov->batch);
  void* p[] = {ov->Z, ov->y, ov->w, ov->y0, ov->q, ov->part};
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
  const int rc = zolotarev_coeffs(lmin / lmax, ov->order, ov->z);
  if (rc) return rc;
  ov->ready = true;
  return QED3_OK;
}

// all poles in one batched launch: Z_m = (D^dag D + lmax^2 sigma_m)^{-1} rhs
static int pole_solves(qed3_overlap_s* ov, const double* rhs, double tol, qed3_solve_report* worst, cudaStream_t st) {
  const int np = ov->order / 2;
  std::vector<double> shifts(np);
  for (int m = 1; m <= np; m++) shifts[m - 1] = ov->lmax * ov->lmax * (-ov->z.k * ov->z.k / ov->z.cp[m]);
  double* xs[1] = {ov->Z};
  const double* bs[1] = {rhs};
  const double* sh[1] = {shifts.data()};
  qed3_solve_params p{tol, 0, ov->prec, 0.1, 0.0, QED3_SOLVE_BCAST_B};
  std::vector<qed3_solve_report> reps(np);
  float ms = 0;
  const int rc = batch_solve(ov->batch, xs, bs, sh, &p, reps.data(), &ms, st);
  if (rc) return rc;
  qed3_solve_report w{};
  for (auto& r : reps) {
    if (r.status != QED3_OK) w.status = r.status;
    w.iters = std::max(w.iters, r.iters);
    w.reliable_updates = std::max(w.reliable_updates, r.reliable_updates);
    w.true_rel_res = std::max(w.true_rel_res, r.true_rel_res);
  }
  w.ms = ms;
  if (worst) *worst = w;
  return w.status == QED3_OK ? QED3_OK : fail(w.status, "a pole solve did not converge");
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
    if ((rc = pole_solves(ov, in, tol, &r1, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), ov->Z, in, ov->y, st))) return rc;  // y = xi + sum A l2 z
    if ((rc = dirac_apply_ref(d, QED3_OP_D, ov->w, ov->y, st))) return rc;          // w = D y
  }
  if (adj) {
    if ((rc = dirac_apply_ref(d, QED3_OP_DDAG, ov->y0, in, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0 / ov->lmax, ov->y0, 0.0, ov->y0, ov->y0, st))) return rc;  // y0 = D^dag xi / lmax
    if ((rc = pole_solves(ov, ov->y0, tol, &r2, st))) return rc;
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

}  // namespace qed3

namespace qed3 {
int overlap_info(const qed3_overlap_s* ov, double* lmin, double* lmax, double* k, double* delta, int* np) {
  if (lmin) *lmin = ov->lmin;
  if (lmax) *lmax = ov->lmax;
  if (k) *k = ov->ready ? ov->z.k : 0.0;
  if (delta) *delta = ov->ready ? (ov->z.lambda_inv - 1.0) / (ov->z.lambda_inv + 1.0) : 0.0;
  if (np) *np = ov->order / 2;
  return QED3_OK;
}
}  // namespace qed3
