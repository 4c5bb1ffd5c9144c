// Multi-shift CG: (D^dag D + sigma_m) x_m = b for all shifts in ONE Krylov space.
//
// Replaces the per-pole CG solves of Overlap (src/both_3d/overlap.h:309-332,
// 343-358, 404-411: one MatPoly::solve per Zolotarev pole, each its own Krylov
// space) by the shifted-CG recurrence (Frommer; Jegerlehner): the base system
// is the smallest shift (the worst-conditioned pole, which converges last);
// every other shift follows with scalar recurrences
//   zeta'_m = zeta_m zold_m a_old / (a b_old (zold_m - zeta_m) + zold_m a_old (1 + d_m a)),
//   a_m = a zeta'_m / zeta_m,  b_m = b (zeta'_m / zeta_m)^2,
//   x_m += a_m p_m,  p_m = zeta'_m r' + b_m p_m,      (d_m = sigma_m - sigma_base)
// and its residual is zeta_m r (collinear with the base residual), so shift m
// stops (and its x_m freezes) as soon as |zeta_m|^2 |r|^2 < tol^2 |b|^2.  One
// D^dag D product per iteration serves all shifts.  FP64 throughout: the
// shifted recurrences need the residuals to stay collinear, which mixed
// precision with reliable updates breaks.
//
// Same persistent skeleton as the register-resident CG (solver_v2.cu): one
// block per SM, two grid barriers per iteration (t = D r + b t gathers r, q =
// D^dag t gathers t), reductions on the barriers; the shift scalars are
// computed identically by every block; x_m and p_m (FP64, internal order)
// live in global memory, read and written once per active shift and site per
// iteration.

#include <cmath>
#include <vector>

#include "batched_impl.h"
#include "blas_impl.h"
#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"
#include "mshift_impl.h"
#include "v2_common.cuh"

namespace qed3 {

struct MsArgs {
  int Ns, ns;
  const int* nbr;
  const M64* H;
  const M64* Hd;
  const double* diag;
  const S64* b;
  S64* X;  // [ns][Ns]
  S64* Pm; // [ns][Ns]
  S64* halo_r;
  S64* halo_t;
  double* partials;
  GridBar2* bar;
  double* scal;  // [0] iterations, [1] |b|^2, [2] status, [3 + m] iteration at which shift m stopped
  double sig_b;
  double dsig[kMsMaxShifts];  // sigma_m - sigma_base >= 0
  double tol2;
  int maxiter;
  long long spin_limit;
};

template <int SPT>
__global__ void __launch_bounds__(640, 1) k_mscg(MsArgs a) {
  __shared__ double sh[32 * 3 + 64 + 8];
  __shared__ double zeta[kMsMaxShifts], zold[kMsMaxShifts], zn[kMsMaxShifts], am[kMsMaxShifts], bm[kMsMaxShifts];
  __shared__ int act[kMsMaxShifts];
  __shared__ int nact;
  const int Ns = a.Ns, ns = a.ns;
  const int T = blockDim.x;
  const int base = blockIdx.x * T * SPT + threadIdx.x;
  int own[SPT];
  bool val[SPT];
  int jj[SPT][3];
  Sp64 r[SPT], p[SPT], t[SPT];
  const Sp64 z64{make_double2(0, 0), make_double2(0, 0)};
  double v1[1] = {0.0};
#pragma unroll
  for (int k = 0; k < SPT; k++) {
    const int i = base + k * T;
    own[k] = i;
    val[k] = i < Ns;
    r[k] = p[k] = t[k] = z64;
    jj[k][0] = jj[k][1] = jj[k][2] = 0;
    if (val[k]) {
      jj[k][0] = __ldg(a.nbr + i);
      jj[k][1] = __ldg(a.nbr + Ns + i);
      jj[k][2] = __ldg(a.nbr + 2 * Ns + i);
      r[k] = ld64(a.b, i);
      v1[0] += n2(r[k]);
      hs64(a.halo_r, i, r[k]);
      for (int m = 0; m < ns; m++) {
        hs64(a.X + size_t(m) * Ns, i, z64);
        hs64(a.Pm + size_t(m) * Ns, i, r[k]);
      }
    }
  }
  if (threadIdx.x < ns) {
    zeta[threadIdx.x] = zold[threadIdx.x] = 1.0;
    act[threadIdx.x] = 1;
  }
  unsigned int epoch = 0;
  int parity = 0;
  v2_publish<1>(v1, a.partials, parity, sh);
  if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
  {
    double tot[1];
    v2_total<1>(a.partials, parity, tot, sh);
    parity ^= 1;
    const double bnorm2 = tot[0];
    double rho = bnorm2, beta = 0.0, a_old = 1.0, b_old = 0.0;
    int iter = 0, status = QED3_ERR_NOCONV;
    const double s = a.sig_b;
    if (bnorm2 == 0.0) {  // x_m = 0 already
      status = QED3_OK;
      if (threadIdx.x < ns && blockIdx.x == 0) a.scal[3 + threadIdx.x] = 0;
      goto finish;
    }
    while (true) {
      // ---- phase A: t = D r + beta t, p = r + beta p ------------------------------------
      {
        double v[1] = {0.0};
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const Sp64 dr = stencil64(own[k], Ns, jj[k], a.H, a.diag, r[k], a.halo_r);
          t[k].s0 = cadd(dr.s0, cscale(beta, t[k].s0));
          t[k].s1 = cadd(dr.s1, cscale(beta, t[k].s1));
          p[k].s0 = cadd(r[k].s0, cscale(beta, p[k].s0));
          p[k].s1 = cadd(r[k].s1, cscale(beta, p[k].s1));
          hs64(a.halo_t, own[k], t[k]);
          v[0] += n2(t[k]) + s * n2(p[k]);
        }
        v2_publish<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double gam[1];
      v2_total<1>(a.partials, parity, gam, sh);
      parity ^= 1;
      const double alpha = rho / gam[0];
      // ---- phase B: r -= alpha (D^dag t + s p) ---------------------------------------------
      {
        double v[1] = {0.0};
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const Sp64 q = stencil64(own[k], Ns, jj[k], a.Hd, a.diag, t[k], a.halo_t);
          r[k].s0 = csub(r[k].s0, cscale(alpha, cadd(q.s0, cscale(s, p[k].s0))));
          r[k].s1 = csub(r[k].s1, cscale(alpha, cadd(q.s1, cscale(s, p[k].s1))));
          hs64(a.halo_r, own[k], r[k]);
          v[0] += n2(r[k]);
        }
        v2_publish<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double rn[1];
      v2_total<1>(a.partials, parity, rn, sh);
      parity ^= 1;
      iter++;
      const double rho_new = rn[0];
      beta = rho_new / rho;
      // ---- shift scalars (identical in every block) ---------------------------------------
      if (threadIdx.x < ns && act[threadIdx.x]) {
        const int m = threadIdx.x;
        const double z = zeta[m], zo = zold[m];
        const double den = alpha * b_old * (zo - z) + zo * a_old * (1.0 + a.dsig[m] * alpha);
        const double znew = z * zo * a_old / den;
        zn[m] = znew;
        am[m] = alpha * znew / z;
        bm[m] = beta * (znew / z) * (znew / z);
      }
      __syncthreads();
      // ---- shifted solutions and directions -----------------------------------------------
      for (int m = 0; m < ns; m++) {
        if (!act[m]) continue;
        const double amm = am[m], bmm = bm[m], znm = zn[m];
        S64* Xm = a.X + size_t(m) * Ns;
        S64* Pmm = a.Pm + size_t(m) * Ns;
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const int i = own[k];
          Sp64 xm = hl64(Xm, i);
          Sp64 pm = hl64(Pmm, i);
          xm.s0 = cadd(xm.s0, cscale(amm, pm.s0));
          xm.s1 = cadd(xm.s1, cscale(amm, pm.s1));
          pm.s0 = cadd(cscale(znm, r[k].s0), cscale(bmm, pm.s0));
          pm.s1 = cadd(cscale(znm, r[k].s1), cscale(bmm, pm.s1));
          hs64(Xm, i, xm);
          hs64(Pmm, i, pm);
        }
      }
      __syncthreads();  // every read of the scalars is done before they change
      if (threadIdx.x == 0) nact = 0;
      __syncthreads();
      if (threadIdx.x < ns && act[threadIdx.x]) {
        const int m = threadIdx.x;
        zold[m] = zeta[m];
        zeta[m] = zn[m];
        // residual of shift m = zeta_m r
        if (zn[m] * zn[m] * rho_new < a.tol2 * bnorm2 || !isfinite(zn[m])) {
          act[m] = 0;
          if (blockIdx.x == 0) a.scal[3 + m] = iter;
        } else {
          atomicAdd(&nact, 1);
        }
      }
      a_old = alpha;
      b_old = beta;
      rho = rho_new;
      __syncthreads();
      if (nact == 0) {
        status = QED3_OK;
        break;
      }
      if (iter >= a.maxiter || !isfinite(rho_new)) {
        if (threadIdx.x < ns && act[threadIdx.x] && blockIdx.x == 0) a.scal[3 + threadIdx.x] = iter;
        break;
      }
    }
  finish:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.scal[0] = iter;
      a.scal[1] = bnorm2;
      a.scal[2] = status;
    }
    return;
  }
timeout:
  if (blockIdx.x == 0 && threadIdx.x == 0) a.scal[2] = QED3_ERR_TIMEOUT;
}

template <int SPT>
static int ms_occupancy(int T, int* per_sm) {
  QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_mscg<SPT>, T, 0));
  return QED3_OK;
}

// x_ref[m] (device, reference order, ns vectors back to back) =
// (D^dag D + shifts[m])^{-1} b_ref; X, Pm: device scratch of ns internal FP64
// fields each.  reps[m]: iterations at which shift m stopped, the FP64 true
// residual ||b - (D^dag D + shift_m) x_m|| / ||b||, status.
int mshift_solve(qed3_dirac_s* d, int ns, const double* shifts, const double* b_ref, double* x_ref, S64* X, S64* Pm,
                 double tol, int maxiter, qed3_solve_report* reps, float* ms_out, cudaStream_t st, bool certify_all) {
  if (ns < 1 || ns > kMsMaxShifts) return fail(QED3_ERR_ARG, "multi-shift: 1..64 shifts");
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  int rc = ensure_work(d);
  if (rc) return rc;
  SolverWork& w = d->work;
  const int Ns = d->Ns;
  double smin = shifts[0];
  for (int m = 0; m < ns; m++) {
    if (!(shifts[m] >= 0.0)) return fail(QED3_ERR_ARG, "multi-shift: shifts must be >= 0");
    smin = std::min(smin, shifts[m]);
  }
  // grid: every site owned by one thread (the register-resident layout)
  int grid = 0, T = 0, spt = 0;
  for (int sp : {1, 2}) {
    const long long per_block = (Ns + d->sm_count - 1) / d->sm_count;
    const int Tt = int(((per_block + sp - 1) / sp + 31) / 32 * 32);
    if (Tt > 640) continue;
    int per_sm = 0;
    if ((sp == 1 ? ms_occupancy<1>(Tt, &per_sm) : ms_occupancy<2>(Tt, &per_sm)) || per_sm < 1) continue;
    const int G = int((Ns + (long long)Tt * sp - 1) / ((long long)Tt * sp));
    if (G > per_sm * d->sm_count) continue;
    grid = G;
    T = std::max(32, Tt);
    spt = sp;
    break;
  }
  if (!grid) return fail(QED3_ERR_ARG, "multi-shift: lattice too large for the register-resident layout");
  if ((rc = field_import(d, QED3_PREC_F64, w.b, b_ref, 1, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(w.bar2, 0, sizeof(GridBar2), st));
  MsArgs a{};
  a.Ns = Ns;
  a.ns = ns;
  a.nbr = d->lat->dev.nbr;
  a.H = d->H;
  a.Hd = d->Hd;
  a.diag = d->diag;
  a.b = w.b;
  a.X = X;
  a.Pm = Pm;
  a.halo_r = reinterpret_cast<S64*>(w.r);
  a.halo_t = reinterpret_cast<S64*>(w.t);
  a.partials = w.partials;
  a.bar = w.bar2;
  a.sig_b = smin;
  for (int m = 0; m < ns; m++) a.dsig[m] = shifts[m] - smin;
  a.tol2 = tol * tol;
  a.maxiter = maxiter;
  a.spin_limit = 4000000LL;
  double* scal = nullptr;
  QED3_CUDA_TRY(cudaMalloc(&scal, (3 + kMsMaxShifts) * sizeof(double)));
  QED3_CUDA_TRY(cudaMemsetAsync(scal, 0, (3 + kMsMaxShifts) * sizeof(double), st));
  a.scal = scal;
  void* kargs[] = {&a};
  QED3_CUDA_TRY(cudaEventRecord(w.e0, st));
  const void* fn = spt == 1 ? (const void*)k_mscg<1> : (const void*)k_mscg<2>;
  rc = QED3_OK;
  if (cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(T), kargs, 0, st) != cudaSuccess)
    rc = fail(QED3_ERR_CUDA, "multi-shift launch failed");
  if (!rc && cudaEventRecord(w.e1, st) != cudaSuccess) rc = fail(QED3_ERR_CUDA, "event record failed");
  std::vector<double> hs(3 + kMsMaxShifts);
  if (!rc && (cudaMemcpyAsync(hs.data(), scal, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess))
    rc = fail(QED3_ERR_CUDA, "multi-shift read-back failed");
  cudaFree(scal);
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, w.e0, w.e1);
  if (int(hs[2]) == QED3_ERR_TIMEOUT) return fail(QED3_ERR_TIMEOUT, "grid barrier timed out in the multi-shift kernel");
  // solutions to reference order, then the FP64 certificate of every shift
  if ((rc = field_export(d, QED3_PREC_F64, x_ref, X, ns, st))) return rc;
  if (!certify_all && int(hs[2]) == QED3_OK) {
    if (ms_out) *ms_out = ms;
    for (int m = 0; m < ns; m++) {
      qed3_solve_report r{};
      r.iters = int(hs[3 + m]);
      r.true_rel_res = -1.0;  // not recomputed
      r.status = QED3_OK;
      r.ms = ms;
      if (reps) reps[m] = r;
    }
    return QED3_OK;
  }
  const double bb = hs[1];
  const long long nd = 4LL * Ns;
  double* q = reinterpret_cast<double*>(w.xhi2);  // scratch, one reference-order vector
  std::vector<double> res2(ns, 0.0);
  auto certify = [&](int m) -> int {
    if (bb == 0) return QED3_OK;
    const double* xm = x_ref + size_t(m) * nd;
    int e = dirac_apply_ref(d, QED3_OP_DDAGD, q, xm, st);
    if (!e) e = ms_residual(nd, q, xm, shifts[m], b_ref, w.partials, &res2[m], st);
    return e;
  };
  for (int m = 0; m < ns; m++)
    if ((rc = certify(m))) return rc;
  // Defect correction for shifts whose true residual the FP64 recurrence could
  // not bring below tol (its recursive and true residuals part by ~kappa eps):
  // delta_m = (D^dag D + s_m)^{-1} (b - (D^dag D + s_m) x_m) by one batched
  // mixed-precision launch to the modest relative accuracy needed, x_m += delta_m.
  for (int pass = 0; pass < 3 && bb > 0; pass++) {
    std::vector<int> bad;
    double need = 1.0;
    for (int m = 0; m < ns; m++)
      if (res2[m] > tol * tol * bb) {
        bad.push_back(m);
        need = std::min(need, 0.3 * tol * std::sqrt(bb / res2[m]));
      }
    if (bad.empty()) break;
    const int nb = int(bad.size());
    double *R = nullptr, *Dl = nullptr;
    if (cudaMalloc(&R, size_t(nb) * nd * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&Dl, size_t(nb) * nd * sizeof(double)) != cudaSuccess) {
      if (R) cudaFree(R);
      return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
    }
    std::vector<double> bsh(nb);
    for (int k = 0; k < nb && !rc; k++) {
      const int m = bad[k];
      bsh[k] = shifts[m];
      const double* xm = x_ref + size_t(m) * nd;
      double* rk = R + size_t(k) * nd;
      rc = dirac_apply_ref(d, QED3_OP_DDAGD, q, xm, st);  // r = b - q - s x
      if (!rc) rc = vec_axpby(nd, 1.0, b_ref, -1.0, q, rk, st);
      if (!rc) rc = vec_axpby(nd, 1.0, rk, -shifts[m], xm, rk, st);
    }
    qed3_batch_s* bt = nullptr;
    qed3_dirac_s* ops[1] = {d};
    const int nr[1] = {nb};
    if (!rc) rc = batch_create(1, ops, nr, QED3_PREC_F32, 0, 0, &bt);
    if (!rc) {
      double* xs[1] = {Dl};
      const double* bs[1] = {R};
      const double* sh[1] = {bsh.data()};
      qed3_solve_params p{std::max(need, 1e-7), 0, QED3_PREC_F32, 0.1, 0.0, 0};
      std::vector<qed3_solve_report> br(nb);
      float bms = 0;
      rc = batch_solve(bt, xs, bs, sh, &p, br.data(), &bms, st);
      ms += bms;
    }
    for (int k = 0; k < nb && !rc; k++) {
      const int m = bad[k];
      rc = vec_axpby(nd, 1.0, x_ref + size_t(m) * nd, 1.0, Dl + size_t(k) * nd, x_ref + size_t(m) * nd, st);
      if (!rc) rc = certify(m);
    }
    if (bt) batch_destroy(bt);
    cudaFree(R);
    cudaFree(Dl);
    if (rc) return rc;
  }
  if (ms_out) *ms_out = ms;
  for (int m = 0; m < ns; m++) {
    qed3_solve_report r{};
    r.iters = int(hs[3 + m]);
    r.reliable_updates = 0;
    r.true_rel_res = bb > 0 ? std::sqrt(res2[m] / bb) : 0.0;
    r.status = (r.true_rel_res <= tol * 1.05 || bb == 0) ? QED3_OK : QED3_ERR_NOCONV;
    r.ms = ms;
    if (reps) reps[m] = r;
  }
  return QED3_OK;
}

// |b - (q + s x)|^2 over nd doubles (reference order): the certificate
__global__ void k_ms_residual(long long nc, const double2* __restrict__ q, const double2* __restrict__ x, double s,
                              const double2* __restrict__ b, double* __restrict__ part) {
  __shared__ double shr[32];
  double v[1] = {0.0};
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nc; k += (long long)gridDim.x * blockDim.x) {
    const double2 e = make_double2(b[k].x - q[k].x - s * x[k].x, b[k].y - q[k].y - s * x[k].y);
    v[0] += e.x * e.x + e.y * e.y;
  }
  block_sum<1>(v, shr);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

int ms_residual(long long nd, const double* q, const double* x, double s, const double* b, double* part, double* out,
                cudaStream_t st) {
  const int blocks = 256;
  k_ms_residual<<<blocks, 256, 0, st>>>(nd / 2, reinterpret_cast<const double2*>(q), reinterpret_cast<const double2*>(x),
                                         s, reinterpret_cast<const double2*>(b), part);
  QED3_CUDA_TRY(cudaGetLastError());
  std::vector<double> h(blocks);
  QED3_CUDA_TRY(cudaMemcpyAsync(h.data(), part, blocks * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  double acc = 0;
  for (double v : h) acc += v;
  *out = acc;
  return QED3_OK;
}

}  // namespace qed3
