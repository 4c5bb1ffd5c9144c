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
#include "lowmodes_impl.h"
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
  bool certify_poles = true;         // FP64 true residual of every pole after each multi-shift solve
  double mass = 0.0;                 // D(m) = (1 - m/2) D_ov + m
  double* Z = nullptr;     // [npoles][2 Ns] complex
  double* y = nullptr;     // [2 Ns] complex
  double* w = nullptr;
  double* y0 = nullptr;
  double* q = nullptr;
  double* part = nullptr;  // reduction scratch
  // force: second pole set and internal-order copies; outer solve: CG vectors
  double* Yp = nullptr;    // [npoles][2 Ns] complex
  double* fi = nullptr;    // [4 npoles + 2][Ns] internal-order two-spinors (4 doubles per site)
  double *sr = nullptr, *sp = nullptr, *sq = nullptr, *se = nullptr, *sb = nullptr;
  // multi-shift scratch (internal-order FP64 fields, [npoles][Ns] each)
  qed3::S64* msX = nullptr;
  qed3::S64* msP = nullptr;
  // low-mode projection: nev eigenvectors h_i of H = gamma5 D / lambda_max
  // (orthonormal, reference order), their eigenvalues mu_i, and the bounds
  // before the projection
  int nev = 0;
  double* lm_h = nullptr;  // [nev][2 Ns] complex
  double* lm_t = nullptr;  // [2][2 Ns] complex scratch
  std::vector<double> lm_mu;
  double lm_res = 0, lm_theta_next = 0, lmin_full = 0;
  int lm_steps = 0;
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
  void* p[] = {ov->Z,  ov->y,  ov->w,   ov->y0,  ov->q,   ov->part, ov->Yp,
               ov->fi, ov->sr, ov->sp,  ov->sq,  ov->msX, ov->msP,  ov->lm_h, ov->lm_t, ov->se, ov->sb};
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
  ov->lmin = ov->lmin_full = lmin;
  ov->lmax = lmax;
  ov->nev = 0;  // new bounds (new links): a projection must be recomputed
  int rc = zolotarev_coeffs(lmin / lmax, ov->order, ov->z);
  if (rc) return rc;
  if ((rc = ov_split(ov))) return rc;
  ov->ready = true;
  return QED3_OK;
}

// Low-mode projection of the sign function.  With h_i the nev eigenvectors
// of H = gamma5 D / lambda_max nearest zero (eigenvalues mu_i):
//   sign(H) = sum_i sign(mu_i) h_i h_i^dag + H r(H^2) (1 - P),  P = sum_i h_i h_i^dag,
// so D_ov = 1 + gamma5 sign(H) becomes
//   D_ov xi     = xi + gamma5 sum_i s_i h_i <h_i, xi> + X r(X^dag X) (1 - P) xi
//   D_ov^dag xi = xi + sum_i s_i h_i <h_i, gamma5 xi> + r(X^dag X) (1 - P) X^dag xi
// (P commutes with X^dag X = H^2), and the Zolotarev range starts at the
// (nev+1)-th |mu| instead of the lowest.  The h_i come from Lanczos on D^dag D
// (lowmodes.cu) followed by Rayleigh-Ritz with H in their span.  The
// reference's Overlap has no projection (src/both_3d/overlap.h:207-306); it
// is an addition for the near-zero modes of H_W at M5 < 0.
int overlap_project_low_modes(qed3_overlap_s* ov, int nev, double tol, int maxsteps, double margin,
                              cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_update first: the projection keeps lambda_max");
  if (nev < 0 || nev > kMaxLowModes) return fail(QED3_ERR_ARG, "low modes: nev must be in [0, 256]");
  qed3_dirac_s* d = ov->d;
  const long long nd = 4LL * d->Ns, nc = nd / 2;
  if (ov->lm_h) cudaFree(ov->lm_h);
  ov->lm_h = nullptr;
  ov->nev = 0;
  ov->lm_mu.clear();
  ov->lm_res = ov->lm_theta_next = 0;
  ov->lm_steps = 0;
  int rc;
  if (nev == 0) {
    ov->lmin = ov->lmin_full;
    if ((rc = zolotarev_coeffs(ov->lmin / ov->lmax, ov->order, ov->z))) return rc;
    return ov_split(ov);
  }
  if (!ov->lm_t) QED3_CUDA_TRY(cudaMalloc(&ov->lm_t, 2 * size_t(nd) * sizeof(double)));
  double* Y = nullptr;
  std::vector<double> th;
  double thn = 0, thmax = 0, res = 0;
  int steps = 0;
  rc = lanczos_lowmodes(
      nd, [&](double* o, const double* v) { return dirac_apply_ref(d, QED3_OP_DDAGD, o, v, st); }, nev, tol,
      maxsteps, &Y, th, &thn, &thmax, &res, &steps, st);
  if (rc) return rc;
  auto body = [&]() -> int {
    // Rayleigh-Ritz with H = gamma5 D / lmax in span{y_i}
    double* t = ov->lm_t;
    std::vector<double> G(2 * size_t(nev) * nev);
    int e;
    for (int j = 0; j < nev; j++) {
      if ((e = dirac_apply_ref(d, QED3_OP_D, t, Y + size_t(j) * nd, st)) || (e = chiral(nd, 0, t, t, st))) return e;
      for (int i = 0; i < nev; i++) {
        double re = 0, im = 0;
        if ((e = vec_zdot(nc, Y + size_t(i) * nd, t, ov->part, &re, &im, st))) return e;
        G[2 * (size_t(i) * nev + j)] = re / ov->lmax;
        G[2 * (size_t(i) * nev + j) + 1] = im / ov->lmax;
      }
    }
    for (int i = 0; i < nev; i++)  // hermitian part (rounding)
      for (int j = i; j < nev; j++) {
        const double re = 0.5 * (G[2 * (size_t(i) * nev + j)] + G[2 * (size_t(j) * nev + i)]);
        const double im = 0.5 * (G[2 * (size_t(i) * nev + j) + 1] - G[2 * (size_t(j) * nev + i) + 1]);
        G[2 * (size_t(i) * nev + j)] = G[2 * (size_t(j) * nev + i)] = re;
        G[2 * (size_t(i) * nev + j) + 1] = im;
        G[2 * (size_t(j) * nev + i) + 1] = -im;
      }
    std::vector<double> mu, U;
    hermitian_eig(nev, G, mu, U);
    if (int(mu.size()) != nev) return fail(QED3_ERR_NOCONV, "low modes: Rayleigh-Ritz lost a vector");
    if ((e = modes_rotate(nd, nev, Y, U, st))) return e;
    double worst = 0;  // ||H h_i - mu_i h_i||
    for (int i = 0; i < nev; i++) {
      const double* h = Y + size_t(i) * nd;
      double r2 = 0, im = 0;
      if ((e = dirac_apply_ref(d, QED3_OP_D, t, h, st)) || (e = chiral(nd, 0, t, t, st)) ||
          (e = vec_axpby(nd, 1.0 / ov->lmax, t, -mu[i], h, t, st)) ||
          (e = vec_zdot(nc, t, t, ov->part, &r2, &im, st)))
        return e;
      worst = std::max(worst, std::sqrt(std::max(r2, 0.0)));
    }
    const double knew = std::sqrt(thn) * (1.0 - margin) / ov->lmax;
    if (!(knew > 0 && knew < 1)) return fail(QED3_ERR_NOCONV, "low modes: no spectral gap above the projected modes");
    ov->lmin = knew * ov->lmax;
    if ((e = zolotarev_coeffs(knew, ov->order, ov->z))) return e;
    if ((e = ov_split(ov))) return e;
    ov->lm_h = Y;
    Y = nullptr;
    ov->nev = nev;
    ov->lm_mu = mu;
    ov->lm_res = worst;
    ov->lm_theta_next = thn;
    ov->lm_steps = steps;
    return QED3_OK;
  };
  rc = body();
  if (Y) cudaFree(Y);
  if (rc) {  // back to the unprojected operator
    ov->lmin = ov->lmin_full;
    zolotarev_coeffs(ov->lmin / ov->lmax, ov->order, ov->z);
    ov_split(ov);
  }
  return rc;
}

// The projected-mode part of D_ov (adj = 0) or D_ov^dag (adj = 1) added to out:
//   adj = 0: out += gamma5 sum_i s_i h_i <h_i, xi>;  adj = 1: out += sum_i s_i h_i <h_i, gamma5 xi>.
static int lowmode_part(qed3_overlap_s* ov, int adj, const double* xi, double* out, cudaStream_t st) {
  const long long nd = 4LL * ov->d->Ns;
  double* t = ov->lm_t;
  int e;
  const double* src = xi;
  if (adj) {
    if ((e = chiral(nd, 0, xi, t, st))) return e;
    src = t;
  }
  std::vector<double> c;
  if ((e = modes_coeffs(nd, ov->nev, ov->lm_h, src, ov->part, c, st))) return e;
  for (int i = 0; i < ov->nev; i++) {
    const double sg = ov->lm_mu[i] >= 0 ? 1.0 : -1.0;
    c[2 * i] *= sg;
    c[2 * i + 1] *= sg;
  }
  double* u = ov->lm_t + nd;
  QED3_CUDA_TRY(cudaMemsetAsync(u, 0, nd * sizeof(double), st));
  if ((e = modes_axpy(nd, ov->nev, ov->lm_h, c, u, u, st))) return e;
  if (!adj && (e = chiral(nd, 0, u, u, st))) return e;
  return vec_axpby(nd, 1.0, u, 1.0, out, out, st);
}

// v <- (1 - P) v
static int lowmode_deflate(qed3_overlap_s* ov, double* v, cudaStream_t st) {
  const long long nd = 4LL * ov->d->Ns;
  std::vector<double> c;
  int e = modes_coeffs(nd, ov->nev, ov->lm_h, v, ov->part, c, st);
  if (e) return e;
  for (auto& x : c) x = -x;
  return modes_axpy(nd, ov->nev, ov->lm_h, c, v, v, st);
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
    const int rc = mshift_solve(ov->d, np, shifts.data(), rhs, out, ov->msX, ov->msP, tol, 200000, reps.data(), &ms, st,
                                ov->certify_poles);
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

// The massless products (D_ov, D_ov^dag, D_ov + D_ov^dag).
static int overlap_apply_massless(qed3_overlap_s* ov, int op, double* out, const double* in, double tol,
                                  qed3_solve_report* rep, cudaStream_t st) {
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
  const bool proj = ov->nev > 0;
  if (mult) {
    const double* src = in;
    if (proj) {  // the rational part acts on (1 - P) xi
      QED3_CUDA_TRY(cudaMemcpyAsync(ov->q, in, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if ((rc = lowmode_deflate(ov, ov->q, st))) return rc;
      src = ov->q;
    }
    if ((rc = pole_solves(ov, src, ov->Z, tol, &r1, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), ov->Z, src, ov->y, st))) return rc;  // y = xi + sum A l2 z
    if ((rc = dirac_apply_ref(d, QED3_OP_D, ov->w, ov->y, st))) return rc;           // w = D y
  }
  if (adj) {
    if ((rc = dirac_apply_ref(d, QED3_OP_DDAG, ov->y0, in, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0 / ov->lmax, ov->y0, 0.0, ov->y0, ov->y0, st))) return rc;  // y0 = D^dag xi / lmax
    if (proj && (rc = lowmode_deflate(ov, ov->y0, st))) return rc;
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
  if (proj) {
    if (mult && (rc = lowmode_part(ov, 0, in, out, st))) return rc;
    if (adj && (rc = lowmode_part(ov, 1, in, out, st))) return rc;
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

// With a mass m: D(m) = (1 - m/2) D_ov + m, and by the Ginsparg-Wilson
// relation D_ov^dag D_ov = D_ov + D_ov^dag,
//   D(m)^dag D(m) = (1 - m^2/4) (D_ov + D_ov^dag) + m^2.
int overlap_apply(qed3_overlap_s* ov, int op, double* out, const double* in, double tol, qed3_solve_report* rep,
                  cudaStream_t st) {
  int rc = overlap_apply_massless(ov, op, out, in, tol, rep, st);
  if (rc || ov->mass == 0.0) return rc;
  const long long nd = 4LL * ov->d->Ns;
  const double m = ov->mass;
  if (op == QED3_OP_D || op == QED3_OP_DDAG) return vec_axpby(nd, 1.0 - 0.5 * m, out, m, in, out, st);
  return vec_axpby(nd, 1.0 - 0.25 * m * m, out, m * m, in, out, st);
}

int overlap_set_mass(qed3_overlap_s* ov, double m) {
  if (!(m >= 0.0 && m < 2.0)) return fail(QED3_ERR_ARG, "overlap mass must be in [0, 2)");
  ov->mass = m;
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
  if (ov->nev > 0)
    return fail(QED3_ERR_STATE, "the overlap force is for the unprojected sign function: switch the low-mode "
                                "projection off (nev = 0) first");
  if (ov->mass != 0.0) return fail(QED3_ERR_STATE, "the overlap force is for the massless operator (mass 0)");
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
// LinOpWrapper of DHD (src/both_3d/prop_nontriv.cu:242-260): x0 = 0, stop on
// the recursive residual; every product is one or two multi-shift pole
// solves.  Options (flags):
//  * QED3_OVSOLVE_CHIRAL: D_ov + D_ov^dag = 2 + gamma5 eps + eps gamma5
//    (eps = gamma5 (D_ov - 1)) commutes with gamma5 for any hermitian eps,
//    and on the chirality-c sector it is 2 P_c D_ov P_c -- one pole solve per
//    iteration instead of two; the sectors are solved one after the other.
// After convergence the true residual ||b - D_ov^dag D_ov x|| is recomputed
// with pole solves to tol_inner; above tol, the CG restarts on that residual
// (at most 4 restarts).  The report: total outer iterations, the certificate,
// reliable_updates = the largest pole iteration count of any product.
int overlap_solve(qed3_overlap_s* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                  int flags, qed3_solve_report* rep, cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_update first");
  const long long nd = 4LL * ov->d->Ns, nc = nd / 2;
  if (!ov->sr) {
    QED3_CUDA_TRY(cudaMalloc(&ov->sr, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->sp, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->sq, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->se, nd * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&ov->sb, nd * sizeof(double)));
  }
  const bool chiral_split = (flags & QED3_OVSOLVE_CHIRAL) != 0;
  cudaEvent_t e0, e1;
  QED3_CUDA_TRY(cudaEventCreate(&e0));
  QED3_CUDA_TRY(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } ev{e0, e1};
  QED3_CUDA_TRY(cudaEventRecord(e0, st));
  int rc, inner_max = 0, it = 0;
  double bb = 0;
  if ((rc = vec_zdot(nc, b, b, ov->part, &bb, nullptr, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(x, 0, nd * sizeof(double), st));
  // the operator of sector c (0: the full D_ov + D_ov^dag)
  // the CG's products skip the per-pole FP64 certificates (the outer
  // certificate below judges the result); poles that stop unconverged are
  // still certified and corrected inside the multi-shift solve
  ov->certify_poles = false;
  struct Restore {
    qed3_overlap_s* o;
    ~Restore() { o->certify_poles = true; }
  } restore{ov};
  auto apply = [&](int c, double* out, const double* v, double tin) -> int {
    qed3_solve_report ir{};
    int e;
    if (c == 0) {
      e = overlap_apply(ov, QED3_OP_DDAGD, out, v, tin, &ir, st);
    } else {  // (1 - m^2/4) 2 P_c D_ov P_c + m^2 on sector c
      const double m = ov->mass;
      e = overlap_apply_massless(ov, QED3_OP_D, out, v, tin, &ir, st);
      if (!e) e = chiral(nd, c, out, out, st);
      if (!e) e = vec_axpby(nd, 2.0 * (1.0 - 0.25 * m * m), out, m * m, v, out, st);
    }
    inner_max = std::max(inner_max, ir.iters);
    return e;
  };
  // CG from zero on A_c e = rhs (ov->sb), e in ov->se, to |r| <= trel |rhs|
  auto cg = [&](int c, double trel, int budget, bool* conv) -> int {
    double rr = 0;
    int e;
    if ((e = vec_zdot(nc, ov->sb, ov->sb, ov->part, &rr, nullptr, st))) return e;
    const double r0 = rr;
    QED3_CUDA_TRY(cudaMemsetAsync(ov->se, 0, nd * sizeof(double), st));
    QED3_CUDA_TRY(cudaMemcpyAsync(ov->sr, ov->sb, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(ov->sp, ov->sb, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    *conv = rr == 0.0;
    for (int k = 0; k < budget && !*conv; k++) {
      if ((e = apply(c, ov->sq, ov->sp, tol_inner))) return e;
      double pq = 0;
      if ((e = vec_zdot(nc, ov->sp, ov->sq, ov->part, &pq, nullptr, st))) return e;
      const double al = rr / pq;
      if ((e = vec_axpby(nd, al, ov->sp, 1.0, ov->se, ov->se, st))) return e;
      if ((e = vec_axpby(nd, -al, ov->sq, 1.0, ov->sr, ov->sr, st))) return e;
      double rn = 0;
      if ((e = vec_zdot(nc, ov->sr, ov->sr, ov->part, &rn, nullptr, st))) return e;
      it++;
      if (!(std::isfinite(rn) && std::isfinite(al))) break;
      if (rn <= trel * trel * r0) {
        *conv = true;
        break;
      }
      if ((e = vec_axpby(nd, 1.0, ov->sr, rn / rr, ov->sp, ov->sp, st))) return e;
      rr = rn;
    }
    return QED3_OK;
  };
  double tr = 0;
  int status = bb == 0.0 ? QED3_OK : QED3_ERR_NOCONV;
  // r = b (x = 0); then restarts on the true residual
  QED3_CUDA_TRY(cudaMemcpyAsync(ov->y0, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double rt = bb;
  for (int restart = 0; restart < 5 && status != QED3_OK && it < maxiter; restart++) {
    const double trel = 0.7 * tol * std::sqrt(bb / rt);  // |r| target relative to this pass's right-hand side
    bool ok = true;
    for (int c : chiral_split ? std::vector<int>{1, -1} : std::vector<int>{0}) {
      if (c == 0) {
        QED3_CUDA_TRY(cudaMemcpyAsync(ov->sb, ov->y0, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
      } else if ((rc = chiral(nd, c, ov->y0, ov->sb, st))) {
        return rc;
      }
      bool conv = false;
      if ((rc = cg(c, chiral_split ? trel / std::sqrt(2.0) : trel, maxiter - it, &conv))) return rc;
      ok = ok && conv;
      if ((rc = vec_axpby(nd, 1.0, ov->se, 1.0, x, x, st))) return rc;
    }
    // certificate: r = b - A x with accurate, certified pole solves
    ov->certify_poles = true;
    rc = overlap_apply(ov, QED3_OP_DDAGD, ov->sq, x, tol_inner, nullptr, st);
    ov->certify_poles = false;
    if (rc) return rc;
    if ((rc = vec_axpby(nd, 1.0, b, -1.0, ov->sq, ov->y0, st))) return rc;
    if ((rc = vec_zdot(nc, ov->y0, ov->y0, ov->part, &tr, nullptr, st))) return rc;
    rt = tr;
    if (tr <= tol * tol * bb) status = QED3_OK;
    else if (!ok && it >= maxiter) break;
  }
  QED3_CUDA_TRY(cudaEventRecord(e1, st));
  QED3_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
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

int overlap_set_pole_solver(qed3_overlap_s* ov, int mode) {
  if (mode != QED3_POLES_MULTISHIFT && mode != QED3_POLES_BATCHED) return fail(QED3_ERR_ARG, "unknown pole solver");
  ov->multishift = mode == QED3_POLES_MULTISHIFT;
  return QED3_OK;
}

int overlap_low_modes_info(const qed3_overlap_s* ov, int* nev, double* max_residual, int* lanczos_steps,
                           double* mu) {
  if (nev) *nev = ov->nev;
  if (max_residual) *max_residual = ov->lm_res;
  if (lanczos_steps) *lanczos_steps = ov->lm_steps;
  if (mu)
    for (int i = 0; i < ov->nev; i++) mu[i] = ov->lm_mu[i];
  return QED3_OK;
}

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
