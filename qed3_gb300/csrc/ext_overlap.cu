// Overlap operator of the S^2 x S^1 Wilson operator: Overlap<DiracExt>
// (src/both_3d/overlap.h:137-390 with WilsonDirac = DiracExt<S2Trivalent,
// DiracS2Dual>, the operator of the reference's IS_OVERLAP builds of hmc.cu
// and prop.cu, src/both_3d/hmc.cu:139-160, src/both_3d/prop.cu:190-215).
//
//   D_ov xi     = xi + (C/lmax) D (xi + sum_m A_m lmax^2 z_m)
//   D_ov^dag xi = xi + C (y0 + sum_m A_m lmax^2 y_m),  y0 = D^dag xi / lmax
//   D_ov^dag D_ov = D_ov + D_ov^dag                     (Overlap::DHD, :363-375)
// with z_m = (D^dag D + lmax^2 sigma_m)^{-1} xi, sigma_m = -k^2/cp_m, k =
// lmin/lmax, the Zolotarev coefficients of zolotarev.cpp (pinned to the
// reference's own build).  All poles come from ONE FP64 multi-shift CG on the
// S^2 x S^1 D^dag D (the reference solves one CG per pole): the base system is
// the smallest shift, the others follow with the shifted-CG scalars (computed
// on the device), all shifts' x_m, p_m updates are one kernel per iteration,
// and chunks of iterations replay as a CUDA graph.  lmin, lmax are
// passed in or come from Lanczos on D^dag D (Ritz values lie inside the
// spectrum; a relative margin widens them).  The outer solve is CG on
// D_ov + D_ov^dag (MatPoly::solve over Overlap::DHD).

#include <algorithm>
#include <cmath>
#include <vector>

#include "blas_impl.h"
#include "device.cuh"
#include "dirac_impl.h"
#include "ext_impl.h"
#include "handles.h"
#include "qed3_internal.h"

struct qed3_overlap_ext_s {
  qed3_dirac_ext_s* e = nullptr;
  int order = 0;
  double lmin = 0, lmax = 0;
  qed3::ZoloCoeffs z;
  bool ready = false;
  double* buf = nullptr;  // Z [np][nd], P [np][nd], r, p, q, y0, y, w, t, then 2048 partials
  double* Yb = nullptr;   // [np][nd] second set of pole solutions (force)
  void* ms = nullptr;     // device state of the multi-shift CG
};

namespace qed3 {

static inline int nblk_o(long long n, int t = 256) { return int((n + t - 1) / t); }

int ext_overlap_create(qed3_dirac_ext_s* e, int order, qed3_overlap_ext_s** out) {
  if (order < 3 || order / 2 > kMaxPoles) return fail(QED3_ERR_ARG, "Zolotarev order must be in [3, 129]");
  auto* ov = new qed3_overlap_ext_s;
  ov->e = e;
  ov->order = order;
  const long long nd = 4LL * e->d2->Ns * e->Nt;
  const int np = order / 2;
  if (cudaMalloc(&ov->buf, (size_t(2 * np + 7) * nd + 2048) * sizeof(double)) != cudaSuccess) {
    delete ov;
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  *out = ov;
  return QED3_OK;
}

void ext_overlap_destroy(qed3_overlap_ext_s* ov) {
  if (!ov) return;
  if (ov->buf) cudaFree(ov->buf);
  if (ov->Yb) cudaFree(ov->Yb);
  if (ov->ms) cudaFree(ov->ms);
  delete ov;
}

// lmin = lmax = 0: sqrt of the extremal eigenvalues of D^dag D by Lanczos to
// rel. tol, widened by margin (lmin (1 - margin), lmax (1 + margin)).
int ext_overlap_update(qed3_overlap_ext_s* ov, double lmin, double lmax, double tol, double margin,
                       cudaStream_t st) {
  qed3_dirac_ext_s* e = ov->e;
  if (!e->links_set) return fail(QED3_ERR_STATE, "call qed3_dirac_ext_set_links first");
  if (!(lmin > 0 && lmax > 0)) {
    const long long nd = 4LL * e->d2->Ns * e->Nt;
    double a = 0, b = 0;
    int steps = 0;
    const int rc = lanczos_extremal(
        nd, [&](double* o, const double* v) { return ext_apply(e, QED3_OP_DDAGD, o, v, st); }, tol > 0 ? tol : 1e-10,
        20000, &a, &b, &steps, st);
    if (rc && rc != QED3_ERR_NOCONV) return rc;
    if (!(a > 0)) return fail(QED3_ERR_NOCONV, "Lanczos gave a non-positive lower bound");
    lmin = std::sqrt(a) * (1.0 - margin);
    lmax = std::sqrt(b) * (1.0 + margin);
  }
  if (!(lmin > 0 && lmin < lmax)) return fail(QED3_ERR_ARG, "need 0 < lambda_min < lambda_max");
  ov->lmin = lmin;
  ov->lmax = lmax;
  const int rc = zolotarev_coeffs(lmin / lmax, ov->order, ov->z);
  if (rc) return rc;
  ov->ready = true;
  return QED3_OK;
}

// ---- multi-shift CG with device-resident scalars ---------------------------
// State: base-system scalars, then per shift zeta, zold, active flag and the
// step coefficients a_m, z_m, b_m (np <= kMaxPoles).  All kernels return at
// once when `done` is set, so a replayed chunk past convergence is a no-op.
struct MsState {
  double rho, alpha, beta, a_old, b_old, done, iters, thr, pq;
  double zeta[kMaxPoles], zold[kMaxPoles], act[kMaxPoles], am[kMaxPoles], zm[kMaxPoles], bm[kMaxPoles];
};
constexpr int kMsParts = 304;

__global__ void k_ms_pq(long long nc, const double2* __restrict__ p, const double2* __restrict__ q,
                        double* __restrict__ part, const MsState* __restrict__ S) {
  if (S->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    const double2 a = p[i], b = q[i];
    v[0] += a.x * b.x + a.y * b.y;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_ms_alpha(const double* __restrict__ part, int np, MsState* __restrict__ S) {
  if (S->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < np; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) S->alpha = S->rho / v[0];
}

// r -= alpha q, partial sums of |r|^2
__global__ void k_ms_r(long long nc, const double2* __restrict__ q, double2* __restrict__ r, double* __restrict__ part,
                       const MsState* __restrict__ S) {
  if (S->done != 0.0) return;
  __shared__ double sh[32];
  const double al = S->alpha;
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    double2 rr = r[i];
    const double2 qq = q[i];
    rr.x -= al * qq.x;
    rr.y -= al * qq.y;
    r[i] = rr;
    v[0] += rr.x * rr.x + rr.y * rr.y;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// |r|^2, beta and every active shift's zeta recurrence (Frommer; Jegerlehner)
__global__ void k_ms_scalars(const double* __restrict__ part, int nparts, int ns, const double* __restrict__ dsig,
                             MsState* __restrict__ S) {
  if (S->done != 0.0) return;
  __shared__ double sh[32];
  __shared__ double rn_s;
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) rn_s = v[0];
  __syncthreads();
  const double rn = rn_s, alpha = S->alpha, beta = rn / S->rho, a_old = S->a_old, b_old = S->b_old;
  const int m = threadIdx.x;
  if (m < ns) {
    if (S->act[m] != 0.0) {
      const double z = S->zeta[m], zo = S->zold[m];
      const double den = alpha * b_old * (zo - z) + zo * a_old * (1.0 + dsig[m] * alpha);
      const double zn = z * zo * a_old / den;
      S->am[m] = alpha * zn / z;
      S->zm[m] = zn;
      S->bm[m] = beta * (zn / z) * (zn / z);
      S->zold[m] = z;
      S->zeta[m] = zn;
      if (zn * zn * rn < S->thr || !isfinite(zn)) S->act[m] = 0.0;
    } else {
      S->am[m] = 0.0;
      S->zm[m] = 0.0;
      S->bm[m] = 1.0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nact = 0;
    for (int k = 0; k < ns; k++) nact += S->act[k] != 0.0;
    S->beta = beta;
    S->a_old = alpha;
    S->b_old = beta;
    S->rho = rn;
    S->iters += 1.0;
    if (!isfinite(rn)) S->done = 2.0;
    // once done is set, k_ms_update_dev (next in stream order) and every later kernel of the
    // iteration return at once, so the step's updates are skipped
    S->pq = nact;
  }
}

// x_m += a_m p_m, p_m = z_m r + b_m p_m for every shift, then p = r + beta p; sets done when no shift is active
__global__ void k_ms_update_dev(long long nd, int ns, const double* __restrict__ r, double* __restrict__ X,
                                double* __restrict__ P, double* __restrict__ p, MsState* __restrict__ S) {
  if (S->done != 0.0) return;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) {
    const double ri = r[i];
    for (int m = 0; m < ns; m++) {
      const size_t o = size_t(m) * nd + i;
      const double pm = P[o];
      X[o] += S->am[m] * pm;
      P[o] = S->zm[m] * ri + S->bm[m] * pm;
    }
    p[i] = ri + S->beta * p[i];
  }
}

__global__ void k_ms_finish(MsState* __restrict__ S) {
  if (S->done == 0.0 && S->pq == 0.0) S->done = 1.0;
}

// (D^dag D + s_m) Z_m = rhs for all poles, s_m = lmax^2 sigma_m: FP64 multi-shift CG
static int ext_pole_solves(qed3_overlap_ext_s* ov, const double* rhs, double tol, int* iters, cudaStream_t st) {
  qed3_dirac_ext_s* e = ov->e;
  const long long nd = 4LL * e->d2->Ns * e->Nt, nc = nd / 2;
  const int np = ov->order / 2;
  double *Z = ov->buf, *P = Z + size_t(np) * nd, *r = P + size_t(np) * nd, *p = r + nd, *q = p + nd;
  double* part = ov->buf + size_t(2 * np + 7) * nd;
  if (!ov->ms) QED3_CUDA_TRY(cudaMalloc(&ov->ms, sizeof(MsState) + kMaxPoles * sizeof(double)));
  MsState* S = reinterpret_cast<MsState*>(ov->ms);
  double* dsig = reinterpret_cast<double*>(S + 1);
  std::vector<double> s(np);
  for (int m = 1; m <= np; m++) s[m - 1] = ov->lmax * ov->lmax * (-ov->z.k * ov->z.k / ov->z.cp[m]);
  const double sb = *std::min_element(s.begin(), s.end());
  std::vector<double> ds(np);
  for (int m = 0; m < np; m++) ds[m] = s[m] - sb;
  int rc;
  double bb = 0, im = 0;
  if ((rc = vec_zdot(nc, rhs, rhs, part, &bb, &im, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(Z, 0, size_t(np) * nd * sizeof(double), st));
  QED3_CUDA_TRY(cudaMemcpyAsync(r, rhs, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(p, rhs, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  for (int m = 0; m < np; m++)
    QED3_CUDA_TRY(cudaMemcpyAsync(P + size_t(m) * nd, rhs, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  MsState h{};
  h.rho = bb;
  h.a_old = 1.0;
  h.b_old = 0.0;
  h.done = bb > 0 ? 0.0 : 1.0;
  h.thr = tol * tol * bb;
  h.pq = np;
  for (int m = 0; m < np; m++) {
    h.zeta[m] = h.zold[m] = 1.0;
    h.act[m] = 1.0;
  }
  QED3_CUDA_TRY(cudaMemcpyAsync(S, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(dsig, ds.data(), np * sizeof(double), cudaMemcpyHostToDevice, st));
  const int gblk = int(std::min<long long>(kMsParts, (nc + 255) / 256));
  auto iter = [&](cudaStream_t cs) -> int {
    int c = ext_apply(e, QED3_OP_DDAGD, q, p, cs);
    if (!c) c = vec_axpby(nd, sb, p, 1.0, q, q, cs);
    if (c) return c;
    k_ms_pq<<<gblk, 256, 0, cs>>>(nc, reinterpret_cast<const double2*>(p), reinterpret_cast<const double2*>(q), part, S);
    k_ms_alpha<<<1, 256, 0, cs>>>(part, gblk, S);
    k_ms_r<<<gblk, 256, 0, cs>>>(nc, reinterpret_cast<const double2*>(q), reinterpret_cast<double2*>(r), part, S);
    k_ms_scalars<<<1, 128, 0, cs>>>(part, gblk, np, dsig, S);
    k_ms_update_dev<<<nblk_o(nd), 256, 0, cs>>>(nd, np, r, Z, P, p, S);
    k_ms_finish<<<1, 1, 0, cs>>>(S);
    return QED3_OK;
  };
  const int chunk = 8;
  IterGraph graph;
  const bool use_graph = h.done == 0.0 && graph.build(chunk, iter);
  int launched = 0;
  while (h.done == 0.0 && launched < 200000) {
    if (use_graph) {
      QED3_CUDA_TRY(cudaGraphLaunch(graph.exec, st));
    } else {
      for (int k = 0; k < chunk; k++)
        if ((rc = iter(st))) return rc;
    }
    QED3_CUDA_TRY(cudaGetLastError());
    launched += chunk;
    QED3_CUDA_TRY(cudaMemcpyAsync(&h, S, sizeof(h), cudaMemcpyDeviceToHost, st));
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (iters) *iters = int(h.iters);
  if (h.done != 1.0) return fail(QED3_ERR_NOCONV, "multi-shift CG did not converge");
  return QED3_OK;
}

int ext_overlap_apply(qed3_overlap_ext_s* ov, int op, double* out, const double* in, double tol, int* iters,
                      cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_ext_update first");
  qed3_dirac_ext_s* e = ov->e;
  const long long nd = 4LL * e->d2->Ns * e->Nt;
  const int np = ov->order / 2;
  double *Z = ov->buf, *y0 = Z + size_t(2 * np) * nd + 3 * nd, *y = y0 + nd, *w = y + nd, *t = w + nd;
  const double l2 = ov->lmax * ov->lmax, C = ov->z.C;
  std::vector<double> coef(np);
  for (int m = 1; m <= np; m++) coef[m - 1] = ov->z.A[m] * l2;
  const bool mult = (op == QED3_OP_D || op == QED3_OP_DDAGD || op == QED3_OP_DDDAG);
  const bool adj = (op == QED3_OP_DDAG || op == QED3_OP_DDAGD || op == QED3_OP_DDDAG);
  if (op < QED3_OP_D || op > QED3_OP_DDDAG) return fail(QED3_ERR_ARG, "unknown operator");
  int rc, i1 = 0, i2 = 0;
  if (mult) {
    if ((rc = ext_pole_solves(ov, in, tol, &i1, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), Z, in, t, st))) return rc;  // t = xi + sum A l2 z
    if ((rc = ext_apply(e, QED3_OP_D, w, t, st))) return rc;               // w = D t
  }
  if (adj) {
    if ((rc = ext_apply(e, QED3_OP_DDAG, y0, in, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0 / ov->lmax, y0, 0.0, y0, y0, st))) return rc;
    if ((rc = ext_pole_solves(ov, y0, tol, &i2, st))) return rc;
    if ((rc = vec_pole_sum(nd, np, coef.data(), Z, y0, y, st))) return rc;  // y = y0 + sum A l2 y_m
  }
  if (mult && adj) {
    if ((rc = vec_axpby(nd, C / ov->lmax, w, C, y, t, st))) return rc;
    if ((rc = vec_axpby(nd, 1.0, t, 2.0, in, out, st))) return rc;
  } else if (mult) {
    if ((rc = vec_axpby(nd, C / ov->lmax, w, 1.0, in, out, st))) return rc;
  } else {
    if ((rc = vec_axpby(nd, C, y, 1.0, in, out, st))) return rc;
  }
  if (iters) *iters = std::max(i1, i2);
  return QED3_OK;
}

// MatPoly::solve over Overlap::DHD: CG on D_ov + D_ov^dag (= D_ov^dag D_ov),
// certified by the recomputed FP64 residual.  With prop != 0, the propagator
// of prop.cu's IS_OVERLAP build (src/both_3d/prop.cu:230-268): b is first
// replaced by D_ov^dag b.
int ext_overlap_solve(qed3_overlap_ext_s* ov, double* x, const double* b_in, double tol, double tol_inner,
                      int maxiter, int prop, qed3_solve_report* rep, cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_ext_update first");
  qed3_dirac_ext_s* e = ov->e;
  const long long nd = 4LL * e->d2->Ns * e->Nt, nc = nd / 2;
  double* bufo = nullptr;
  if (cudaMalloc(&bufo, size_t(5) * nd * sizeof(double)) != cudaSuccess) return fail(QED3_ERR_NOMEM, "cudaMalloc");
  double *b = bufo, *r = b + nd, *p = r + nd, *q = p + nd, *tt = q + nd;
  double* part = ov->buf + size_t(2 * (ov->order / 2) + 7) * nd;
  auto body = [&]() -> int {
    int rc;
    if (prop) {
      if ((rc = ext_overlap_apply(ov, QED3_OP_DDAG, b, b_in, tol_inner, nullptr, st))) return rc;
    } else {
      QED3_CUDA_TRY(cudaMemcpyAsync(b, b_in, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    double bb = 0, im = 0;
    if ((rc = vec_zdot(nc, b, b, part, &bb, &im, st))) return rc;
    QED3_CUDA_TRY(cudaMemsetAsync(x, 0, nd * sizeof(double), st));
    QED3_CUDA_TRY(cudaMemcpyAsync(r, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(p, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    double mu = bb;
    int it = 0, status = bb == 0.0 ? QED3_OK : QED3_ERR_NOCONV;
    while (status != QED3_OK && it < maxiter) {
      if ((rc = ext_overlap_apply(ov, QED3_OP_DDAGD, q, p, tol_inner, nullptr, st))) return rc;
      double pq = 0;
      if ((rc = vec_zdot(nc, p, q, part, &pq, &im, st))) return rc;
      const double al = mu / pq;
      if ((rc = vec_axpby(nd, al, p, 1.0, x, x, st)) || (rc = vec_axpby(nd, -al, q, 1.0, r, r, st))) return rc;
      double mn = 0;
      if ((rc = vec_zdot(nc, r, r, part, &mn, &im, st))) return rc;
      it++;
      if (!std::isfinite(mn)) break;
      if (mn < tol * tol * bb) {
        status = QED3_OK;
        break;
      }
      if ((rc = vec_axpby(nd, 1.0, r, mn / mu, p, p, st))) return rc;
      mu = mn;
    }
    double tr = 0;
    if (bb > 0) {
      if ((rc = ext_overlap_apply(ov, QED3_OP_DDAGD, q, x, tol_inner, nullptr, st)) ||
          (rc = vec_axpby(nd, 1.0, b, -1.0, q, tt, st)) || (rc = vec_zdot(nc, tt, tt, part, &tr, &im, st)))
        return rc;
    }
    if (rep) {
      rep->status = status;
      rep->iters = it;
      rep->reliable_updates = 0;
      rep->true_rel_res = bb > 0 ? std::sqrt(tr / bb) : 0.0;
      rep->ms = 0;
    }
    return QED3_OK;
  };
  const int rc = body();
  cudaStreamSynchronize(st);
  cudaFree(bufo);
  return rc;
}

// Overlap pseudofermion force of all links (Overlap::precalc_grad +
// grad_deviceAsyncLaunch, src/both_3d/overlap.h:393-470), F = -2 d/dA Re<eta, D_ov eta>:
//   F = sum_m c_m (Re<D Z'_m, dD Y'_m> + Re<D Y'_m, dD Z'_m>) - 2C/lmax Re<eta, dD w>,
//   c_m = 2 C A_m lmax^2, Z'_m = (D^dag D + lmax^2 s_m)^{-1} eta,
//   Y'_m = (D^dag D + lmax^2 s_m)^{-1} D^dag eta / lmax, w = eta + sum_m A_m lmax^2 Z'_m;
// every Re<a, dD b> is one pass of the link kernels (-2 Re<a, dD b> accumulated with weight).
int ext_overlap_force(qed3_overlap_ext_s* ov, const double* eta, double* F, double tol, int* iters, cudaStream_t st) {
  if (!ov->ready) return fail(QED3_ERR_STATE, "call qed3_overlap_ext_update first");
  qed3_dirac_ext_s* e = ov->e;
  const long long nd = 4LL * e->d2->Ns * e->Nt;
  const int np = ov->order / 2;
  double *Z = ov->buf, *y0 = Z + size_t(2 * np) * nd + 3 * nd, *y = y0 + nd, *w = y + nd, *t = w + nd;
  if (!ov->Yb) QED3_CUDA_TRY(cudaMalloc(&ov->Yb, size_t(np) * nd * sizeof(double)));
  const double l2 = ov->lmax * ov->lmax, C = ov->z.C;
  int rc, i1 = 0, i2 = 0;
  if ((rc = ext_apply(e, QED3_OP_DDAG, y0, eta, st))) return rc;
  if ((rc = vec_axpby(nd, 1.0 / ov->lmax, y0, 0.0, y0, y0, st))) return rc;
  if ((rc = ext_pole_solves(ov, y0, tol, &i2, st))) return rc;
  QED3_CUDA_TRY(cudaMemcpyAsync(ov->Yb, Z, size_t(np) * nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if ((rc = ext_pole_solves(ov, eta, tol, &i1, st))) return rc;
  std::vector<double> coef(np);
  for (int m = 1; m <= np; m++) coef[m - 1] = ov->z.A[m] * l2;
  if ((rc = vec_pole_sum(nd, np, coef.data(), Z, eta, w, st))) return rc;
  // -2C/lmax Re<eta, dD w> = (C/lmax) (-2 Re<eta, dD w>)
  if ((rc = ext_force_bilinear(e, eta, w, C / ov->lmax, 0, F, st))) return rc;
  for (int m = 0; m < np; m++) {
    const double cm = 2.0 * C * ov->z.A[m + 1] * l2;
    const double* Zm = Z + size_t(m) * nd;
    const double* Ym = ov->Yb + size_t(m) * nd;
    if ((rc = ext_apply(e, QED3_OP_D, t, Zm, st)) || (rc = ext_apply(e, QED3_OP_D, y, Ym, st))) return rc;
    if ((rc = ext_force_bilinear(e, t, Ym, -0.5 * cm, 1, F, st)) ||
        (rc = ext_force_bilinear(e, y, Zm, -0.5 * cm, 1, F, st)))
      return rc;
  }
  if (iters) *iters = std::max(i1, i2);
  return QED3_OK;
}

qed3_dirac_ext_s* ext_overlap_operator(qed3_overlap_ext_s* ov) { return ov->e; }

void ext_overlap_info(const qed3_overlap_ext_s* ov, double* lmin, double* lmax, double* k, double* delta) {
  *lmin = ov->lmin;
  *lmax = ov->lmax;
  *k = ov->ready ? ov->z.k : 0.0;
  *delta = ov->ready ? (ov->z.lambda_inv - 1.0) / (ov->z.lambda_inv + 1.0) : 0.0;  // Zolotarev::Delta
}

}  // namespace qed3
