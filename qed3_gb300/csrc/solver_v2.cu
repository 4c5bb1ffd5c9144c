// Persistent CG, register-resident form, for lattices that fit on-chip.
//
// Same iteration as solver.cu (two phases per CG step, FP64 reductions riding
// on the grid barriers, FP64 reliable updates), restructured for the case
// where every site can be owned by one thread for the whole solve (n <= ~98 on
// 152 SMs, e.g. the n=64 workload's 81,920 sites = 152 blocks x 544 threads):
//   * one block per SM, thread t of block b owns sites b*T*SPT + k*T + t;
//   * r, p, t and the solution stay in registers across iterations;
//   * only the two gathered fields travel through memory: each phase stores
//     the owned value of one "halo" field and loads three neighbour values of
//     the other (fp64, fp32, or bf16 copies of fp32 state in the bf16 mode);
//   * hop blocks and ids are read through the read-only path and stay
//     L1-resident (96 B per site and direction);
//   * the grid barrier is the monotonic acq_rel form (grid_sync2).
// A reliable update takes three phases: publish x, t64 = D x, r = b - D^dag t64.

#include <cmath>
#include <string>
#include <type_traits>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"
#include "solver_v2.h"
#include "v2_common.cuh"

namespace qed3 {

template <int P, int SPT>
__global__ void __launch_bounds__(640, 1) k_cg_v2(CgV2Args a) {
  __shared__ double sh[32 * 3 + 64 + 8];
  const int Ns = a.Ns;
  const int T = blockDim.x;
  const int base = blockIdx.x * T * SPT + threadIdx.x;
  constexpr bool mixed = (P != P64);
  using SpT = typename std::conditional<mixed, Sp32, Sp64>::type;

  int own[SPT];
  bool val[SPT];
  int jj[SPT][3];
  SpT r[SPT], p[SPT], t[SPT];
  Sp64 xh[SPT];  // solution (fp64); in mixed mode the part folded at the last update
  Sp32 xl[SPT];  // mixed mode: fp32 increment since the last update
  const Sp64 z64{make_double2(0, 0), make_double2(0, 0)};
  const Sp32 z32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};

  // ---- phase 0: load ids and b, r = b, p = t = x = 0 ------------------------------
  double v1[1] = {0.0};
#pragma unroll
  for (int k = 0; k < SPT; k++) {
    const int i = base + k * T;
    own[k] = i;
    val[k] = i < Ns;
    xh[k] = z64;
    xl[k] = z32;
    if (val[k]) {
      jj[k][0] = __ldg(a.nbr + i);
      jj[k][1] = __ldg(a.nbr + Ns + i);
      jj[k][2] = __ldg(a.nbr + 2 * Ns + i);
      const Sp64 bi = ld64(a.b, i);
      v1[0] += n2(bi);
      if constexpr (mixed) {
        r[k] = Sp32{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
        p[k] = z32;
        t[k] = z32;
        hs32<P>(a.halo_r, i, r[k]);
      } else {
        r[k] = bi;
        p[k] = z64;
        t[k] = z64;
        hs64(reinterpret_cast<S64*>(a.halo_r), i, r[k]);
      }
    } else {
      jj[k][0] = jj[k][1] = jj[k][2] = 0;
      if constexpr (mixed) {
        r[k] = z32; p[k] = z32; t[k] = z32;
      } else {
        r[k] = z64; p[k] = z64; t[k] = z64;
      }
    }
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
    double mu = bnorm2, mu_max = bnorm2, beta = 0.0, mu_true = bnorm2;
    double2 a_r = make_double2(1.0, 0.0);
    int iter = 0, nru = 0, status = QED3_ERR_NOCONV;
    const double s = a.shift;
    if (bnorm2 == 0.0) {
      status = QED3_OK;
      mu_true = 0.0;
      goto finish;
    }
    while (true) {
      // ---- phase A: t = a_r D r + beta t, p = a_r r + beta p -------------------------
      {
        double v[1] = {0.0};
        float vf[1] = {0.f};
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const int i = own[k];
          if constexpr (mixed) {
            const Sp32 dr = stencil32<P>(i, Ns, jj[k], a.H32, a.diag32, r[k], a.halo_r);
            const float2 ar = make_float2(float(a_r.x), float(a_r.y));
            const float bt = float(beta);
            t[k].s0 = cfmaf(ar, dr.s0, make_float2(bt * t[k].s0.x, bt * t[k].s0.y));
            t[k].s1 = cfmaf(ar, dr.s1, make_float2(bt * t[k].s1.x, bt * t[k].s1.y));
            p[k].s0 = cfmaf(ar, r[k].s0, make_float2(bt * p[k].s0.x, bt * p[k].s0.y));
            p[k].s1 = cfmaf(ar, r[k].s1, make_float2(bt * p[k].s1.x, bt * p[k].s1.y));
            hs32<P>(a.halo_t, i, t[k]);
            vf[0] += n2f(t[k]) + float(s) * n2f(p[k]);
          } else {
            const Sp64 dr = stencil64(i, Ns, jj[k], a.H, a.diag, r[k], reinterpret_cast<const S64*>(a.halo_r));
            t[k].s0 = cfma(a_r, dr.s0, cscale(beta, t[k].s0));
            t[k].s1 = cfma(a_r, dr.s1, cscale(beta, t[k].s1));
            p[k].s0 = cfma(a_r, r[k].s0, cscale(beta, p[k].s0));
            p[k].s1 = cfma(a_r, r[k].s1, cscale(beta, p[k].s1));
            hs64(reinterpret_cast<S64*>(a.halo_t), i, t[k]);
            v[0] += n2(t[k]) + s * n2(p[k]);
          }
        }
        if constexpr (mixed) v2_publish_f<1>(vf, a.partials, parity, sh);
        else v2_publish<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double gam[1];
      v2_total<1>(a.partials, parity, gam, sh);
      parity ^= 1;
      const double alpha = mu / gam[0];
      // ---- phase B: q = D^dag t + s p, x += alpha p, r -= alpha q --------------------
      {
        double v[1] = {0.0};
        float vf[1] = {0.f};
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const int i = own[k];
          if constexpr (mixed) {
            const Sp32 q = stencil32<P>(i, Ns, jj[k], a.Hd32, a.diag32, t[k], a.halo_t);
            const float al = float(alpha), sf = float(s);
            r[k].s0 = make_float2(r[k].s0.x - al * (q.s0.x + sf * p[k].s0.x), r[k].s0.y - al * (q.s0.y + sf * p[k].s0.y));
            r[k].s1 = make_float2(r[k].s1.x - al * (q.s1.x + sf * p[k].s1.x), r[k].s1.y - al * (q.s1.y + sf * p[k].s1.y));
            xl[k].s0 = make_float2(xl[k].s0.x + al * p[k].s0.x, xl[k].s0.y + al * p[k].s0.y);
            xl[k].s1 = make_float2(xl[k].s1.x + al * p[k].s1.x, xl[k].s1.y + al * p[k].s1.y);
            hs32<P>(a.halo_r, i, r[k]);
            vf[0] += n2f(r[k]);
          } else {
            const Sp64 q = stencil64(i, Ns, jj[k], a.Hd, a.diag, t[k], reinterpret_cast<const S64*>(a.halo_t));
            r[k].s0 = csub(r[k].s0, cscale(alpha, cadd(q.s0, cscale(s, p[k].s0))));
            r[k].s1 = csub(r[k].s1, cscale(alpha, cadd(q.s1, cscale(s, p[k].s1))));
            xh[k].s0 = cadd(xh[k].s0, cscale(alpha, p[k].s0));
            xh[k].s1 = cadd(xh[k].s1, cscale(alpha, p[k].s1));
            hs64(reinterpret_cast<S64*>(a.halo_r), i, r[k]);
            v[0] += n2(r[k]);
          }
        }
        if constexpr (mixed) v2_publish_f<1>(vf, a.partials, parity, sh);
        else v2_publish<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double mun[1];
      v2_total<1>(a.partials, parity, mun, sh);
      parity ^= 1;
      iter++;
      const double mu_new = mun[0];
      mu_max = fmax(mu_max, mu_new);
      const bool want = !isfinite(mu_new) || !isfinite(alpha) || mu_new < a.tol2 * bnorm2 || iter >= a.maxiter ||
                        (mixed && mu_new < a.delta2 * mu_max);
      if (!want) {
        beta = mu_new / mu;
        a_r = make_double2(1.0, 0.0);
        mu = mu_new;
        continue;
      }
      // ---- R0: fold x, publish it -------------------------------------------------------
#pragma unroll
      for (int k = 0; k < SPT; k++) {
        if (!val[k]) continue;
        if constexpr (mixed) {
          xh[k].s0 = make_double2(xh[k].s0.x + xl[k].s0.x, xh[k].s0.y + xl[k].s0.y);
          xh[k].s1 = make_double2(xh[k].s1.x + xl[k].s1.x, xh[k].s1.y + xl[k].s1.y);
          xl[k] = z32;
        }
        hs64(a.x, own[k], xh[k]);
      }
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R1: t64 = D x ------------------------------------------------------------------
#pragma unroll
      for (int k = 0; k < SPT; k++) {
        if (!val[k]) continue;
        const Sp64 o = stencil64(own[k], Ns, jj[k], a.H, a.diag, xh[k], a.x);
        hs64(a.t64, own[k], o);
      }
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R2: r = b - D^dag t64 - s x;  |r|^2, <r, p> ------------------------------------
      {
        double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const int i = own[k];
          const Sp64 self = hl64(a.t64, i);
          const Sp64 q = stencil64(i, Ns, jj[k], a.Hd, a.diag, self, a.t64);
          const Sp64 bi = ld64(a.b, i);
          Sp64 rt;
          rt.s0 = csub(bi.s0, cadd(q.s0, cscale(s, xh[k].s0)));
          rt.s1 = csub(bi.s1, cadd(q.s1, cscale(s, xh[k].s1)));
          v[0] += n2(rt);
          double2 pv0, pv1;
          if constexpr (mixed) {
            pv0 = make_double2(p[k].s0.x, p[k].s0.y);
            pv1 = make_double2(p[k].s1.x, p[k].s1.y);
            r[k] = Sp32{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
            hs32<P>(a.halo_r, i, r[k]);
          } else {
            pv0 = p[k].s0;
            pv1 = p[k].s1;
            r[k] = rt;
            hs64(reinterpret_cast<S64*>(a.halo_r), i, r[k]);
          }
          v[1] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
          v[2] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
        }
        v2_publish<3>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double tr[3];
      v2_total<3>(a.partials, parity, tr, sh);
      parity ^= 1;
      nru++;
      mu_true = tr[0];
      if (mu_true < a.tol2 * bnorm2) {
        status = QED3_OK;
        break;
      }
      if (iter >= a.maxiter || !isfinite(mu_true)) {
        status = QED3_ERR_NOCONV;
        break;
      }
      beta = mu_true / mu;
      a_r = make_double2(1.0 - beta * tr[1] / mu_true, -beta * tr[2] / mu_true);
      mu = mu_true;
      mu_max = mu_true;
    }
  finish:
    // the converged solution is the one published at the last update
    // (plain fp64 mode: also exact since x is updated in place)
#pragma unroll
    for (int k = 0; k < SPT; k++)
      if (val[k]) hs64(a.x, own[k], xh[k]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.scal[0] = mu_true;
      a.scal[1] = bnorm2;
      a.scal[2] = iter;
      a.scal[3] = nru;
      a.scal[4] = status;
      a.scal[5] = 0;
    }
    return;
  }
timeout:
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[4] = QED3_ERR_TIMEOUT;
    a.scal[5] = 0;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int P, int SPT>
static int v2_occupancy(int T, int* per_sm) {
  QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_cg_v2<P, SPT>, T, 0));
  return QED3_OK;
}

// Picks (blocks, threads, sites per thread) so that every site has an owner
// and every block is resident; returns false when the lattice is too large.
bool cg_v2_plan(int prec, int Ns, int sm_count, int* grid, int* threads, int* spt) {
  for (int s : {1, 2}) {
    const long long per_block = (Ns + sm_count - 1) / sm_count;
    const int T = int(((per_block + s - 1) / s + 31) / 32 * 32);
    if (T > 640) continue;
    int per_sm = 0;
    int rc;
    if (prec == QED3_PREC_F64) rc = s == 1 ? v2_occupancy<P64, 1>(T, &per_sm) : v2_occupancy<P64, 2>(T, &per_sm);
    else if (prec == QED3_PREC_F32) rc = s == 1 ? v2_occupancy<P32, 1>(T, &per_sm) : v2_occupancy<P32, 2>(T, &per_sm);
    else rc = s == 1 ? v2_occupancy<PBF16, 1>(T, &per_sm) : v2_occupancy<PBF16, 2>(T, &per_sm);
    if (rc || per_sm < 1) continue;
    const int G = int((Ns + (long long)T * s - 1) / ((long long)T * s));
    if (G > per_sm * sm_count) continue;
    *grid = G;
    *threads = std::max(32, T);
    *spt = s;
    return true;
  }
  return false;
}

int cg_v2_launch(int prec, int spt, int grid, int threads, CgV2Args& a, cudaStream_t st) {
  void* kargs[] = {&a};
  const void* fn = nullptr;
  if (prec == QED3_PREC_F64) fn = spt == 1 ? (const void*)k_cg_v2<P64, 1> : (const void*)k_cg_v2<P64, 2>;
  else if (prec == QED3_PREC_F32) fn = spt == 1 ? (const void*)k_cg_v2<P32, 1> : (const void*)k_cg_v2<P32, 2>;
  else fn = spt == 1 ? (const void*)k_cg_v2<PBF16, 1> : (const void*)k_cg_v2<PBF16, 2>;
  QED3_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), kargs, 0, st));
  return QED3_OK;
}

}  // namespace qed3
