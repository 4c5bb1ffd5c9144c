// Batched persistent CG: many systems in ONE cooperative launch.
//
// A system is one Wilson-Dirac operator (any lattice size) with R right-hand
// sides that share every stencil read: the three neighbour ids and the three
// hop blocks of a site are loaded once and applied to all R spinors of that
// site (fields are interleaved site-major, [Ns][R]).  Systems may use
// different lattices (multi-lattice), different operators (masses) and a
// shift per right-hand side (the multi-shift refinement of the overlap poles).
//
// Each system runs its own CG state machine
//     INIT -> (A -> B)* -> [R1 -> R2] -> ... -> DONE
// (phases as in solver.cu: A = t = a_r D r + beta t, B = D^dag t and the
// x/r update, R1/R2 = FP64 reliable update / true residual) and every phase
// is followed by one grid-wide barrier, so systems in different phases step in
// lockstep.  The barrier also counts the blocks whose system is DONE: when all
// are, the last arriving block publishes an all-done flag together with the
// new generation and every block leaves the kernel at the same barrier.
// Reductions are per (system, right-hand side), summed in a fixed order by
// every block of the system.
//
// This replaces, for a batch, what the reference does with one MatPoly::solve
// per right-hand side and per pole on OpenMP threads driving CUDA streams
// (src/both_3d/overlap.h:309-332, src/dual/matpoly.h:204-267).
//
// This file holds the static schedule (each system owns a range of blocks,
// re-split after every synchronous solve by the iterations each system took),
// the host side of both schedules and the autotuner; batched_dyn.cu holds the
// dynamic schedule's kernel (warp tiles, no grid barrier).

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "batched_impl.h"
#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"

namespace qed3 {

enum SysState { ST_INIT = 0, ST_A = 1, ST_B = 2, ST_R1 = 3, ST_R2 = 4, ST_DONE = 5 };

// Barrier that also counts "done" arrivals.  count low 16 bits: arrivals,
// high 16 bits: done arrivals.  gen word: generation | all-done << 31.
__device__ __forceinline__ bool grid_sync_vote(GridBar* bar, unsigned int& gen, long long spin_limit, int my_done,
                                               int& all_done) {
  __syncthreads();
  __shared__ int s_ok, s_all;
  if (threadIdx.x == 0) {
    int ok = 1, all = 0;
    __threadfence();
    const unsigned int inc = my_done ? 0x10001u : 1u;
    const unsigned int prev = atomicAdd(&bar->count, inc);
    if ((prev & 0xffffu) == gridDim.x - 1) {
      const unsigned int ndone = (prev >> 16) + (my_done ? 1u : 0u);
      all = (ndone == gridDim.x) ? 1 : 0;
      atomicExch(&bar->count, 0u);
      __threadfence();
      st_release(&bar->gen, ((gen + 1u) & 0x7fffffffu) | (unsigned(all) << 31));
    } else {
      long long spins = 0;
      unsigned int g;
      while (((g = ld_acquire(&bar->gen)) & 0x7fffffffu) == (gen & 0x7fffffffu)) {
        if (ld_volatile_int(&bar->abort)) {
          ok = 0;
          break;
        }
        if (++spins > spin_limit) {
          atomicExch(&bar->abort, 1);
          ok = 0;
          break;
        }
        __nanosleep(40);
      }
      all = int(g >> 31);
    }
    if (ld_volatile_int(&bar->abort)) ok = 0;
    gen = (gen + 1u) & 0x7fffffffu;
    s_ok = ok;
    s_all = all;
  }
  __syncthreads();
  all_done = s_all;
  return s_ok != 0;
}

template <int R>
struct SysScalars {
  double mu[R], mu_max[R], beta[R], bnorm2[R], alpha[R], mu_true[R];
  double2 a_r[R];
  int active[R], status[R], it_done[R];
  int iter, nru, state, xsel;
};

// Block partials: [parity][block][R * 3]
__device__ __forceinline__ double* part_ptr(double* base, int parity, int R3) {
  return base + (size_t(parity) * gridDim.x + blockIdx.x) * R3;
}

// T threads per block.  The scalar state of a system is held per thread, so
// without a register cap the kernel takes 128 registers and four 128-thread
// blocks per SM, and the grid-strided site loops are latency bound.  Capping
// at 64 registers (1024 / T blocks of T threads per SM) for tiles up to 4
// doubles the resident warps (measured the faster shape on the 256-RHS
// multi-lattice batch).
template <int P, int R, int T>
__global__ void __launch_bounds__(T, (R <= 4 ? 1024 / T : 1)) k_batched_cg(BatchArgs a) {
  __shared__ double sh[32 * 3 * R];
  __shared__ double tot[3 * R];
  // ---- my system ----
  const int sidx = a.sys_of_block[blockIdx.x];
  const BatchSys& S = a.sys[sidx];
  const int Ns = S.Ns, nr = S.nrhs;
  const int lb = blockIdx.x - S.blk0, nb = S.blk1 - S.blk0;
  const int tid = lb * blockDim.x + threadIdx.x, nth = nb * blockDim.x;
  const bool mixed = (P != P64);
  using Lo = typename LoField<P == P64 ? P32 : P>::T;

  S64* r64 = reinterpret_cast<S64*>(S.r);
  S64* p64 = reinterpret_cast<S64*>(S.p);
  S64* t64w = reinterpret_cast<S64*>(S.t);
  // mixed modes: r, t are fp32 state; neighbours are read from rh / th, which
  // alias r / t in fp32 mode and are bf16 copies in bf16 mode
  float4* r32 = reinterpret_cast<float4*>(S.r);
  float4* t32 = reinterpret_cast<float4*>(S.t);
  Lo* rh = reinterpret_cast<Lo*>(P == PBF16 ? S.rh : S.r);
  Lo* th = reinterpret_cast<Lo*>(P == PBF16 ? S.th : S.t);
  float4* p32 = reinterpret_cast<float4*>(S.p);
  float4* xlo = reinterpret_cast<float4*>(S.xlo);
  S64* xa = S.xhi;
  S64* xb = S.xhi2;

  SysScalars<R> sc;
  for (int r = 0; r < R; r++) {
    sc.mu[r] = sc.mu_max[r] = sc.beta[r] = sc.bnorm2[r] = sc.alpha[r] = sc.mu_true[r] = 0.0;
    sc.a_r[r] = make_double2(1.0, 0.0);
    sc.active[r] = r < nr;
    sc.status[r] = QED3_ERR_NOCONV;
    sc.it_done[r] = 0;
  }
  sc.iter = 0;
  sc.nru = 0;
  sc.state = ST_INIT;
  sc.xsel = 0;

  unsigned int gen = 0;
  int parity = 0;
  const int R3 = 3 * R;
  const double tol2 = a.tol2, delta2 = a.delta2;

  while (true) {
    double v[3 * R];
#pragma unroll
    for (int q = 0; q < 3 * R; q++) v[q] = 0.0;
    const int st = sc.state;
    // ======================= phase work =======================
    if (st == ST_INIT) {
      for (int i = tid; i < Ns; i += nth) {
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r >= nr) break;
          const size_t e = size_t(i) * R + r;
          const Sp64 bi = ld64(S.b, int(e));
          v[3 * r] += bi.s0.x * bi.s0.x + bi.s0.y * bi.s0.y + bi.s1.x * bi.s1.x + bi.s1.y * bi.s1.y;
          const Sp64 z{make_double2(0, 0), make_double2(0, 0)};
          st64(xa, int(e), z);
          if constexpr (!mixed) {
            st64(r64, int(e), bi);
            st64(p64, int(e), z);
            st64(t64w, int(e), z);
          } else {
            const Sp32 bl{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
            const Sp32 zl{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            st32(r32, int(e), bl);
            st32(t32, int(e), zl);
            if constexpr (P == PBF16) {
              stbf(reinterpret_cast<uint2*>(rh), int(e), bl);
              stbf(reinterpret_cast<uint2*>(th), int(e), zl);
            }
            st32(p32, int(e), zl);
            st32(xlo, int(e), zl);
          }
        }
      }
    } else if (st == ST_A) {
      // mixed: FP32 sums over the thread's sites, FP64 from the block sum on
      float vf[R];
#pragma unroll
      for (int r = 0; r < R; r++) vf[r] = 0.f;
      for (int i = tid; i < Ns; i += nth) {
        const int j0 = __ldg(S.nbr + i), j1 = __ldg(S.nbr + Ns + i), j2 = __ldg(S.nbr + 2 * Ns + i);
        if constexpr (!mixed) {
          const M64 m0 = S.H[i], m1 = S.H[Ns + i], m2 = S.H[2 * Ns + i];
          const double dg = __ldg(S.diag + i);
#pragma unroll
          for (int r = 0; r < R; r++) {
            if (r >= nr || !sc.active[r]) continue;
            const int e = i * R + r;
            const Sp64 self = ld64(r64, e), b0 = ld64(r64, j0 * R + r), b1 = ld64(r64, j1 * R + r),
                       b2 = ld64(r64, j2 * R + r);
            Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
            const M64* ms[3] = {&m0, &m1, &m2};
            const Sp64* bs[3] = {&b0, &b1, &b2};
#pragma unroll
            for (int k = 0; k < 3; k++) {
              o.s0 = cfma(ms[k]->h00, bs[k]->s0, o.s0);
              o.s0 = cfma(ms[k]->h01, bs[k]->s1, o.s0);
              o.s1 = cfma(ms[k]->h10, bs[k]->s0, o.s1);
              o.s1 = cfma(ms[k]->h11, bs[k]->s1, o.s1);
            }
            const Sp64 ti = ld64(t64w, e), pi = ld64(p64, e);
            const double bt = sc.beta[r];
            const double2 ar = sc.a_r[r];
            Sp64 tn, pn;
            tn.s0 = cfma(ar, o.s0, cscale(bt, ti.s0));
            tn.s1 = cfma(ar, o.s1, cscale(bt, ti.s1));
            pn.s0 = cfma(ar, self.s0, cscale(bt, pi.s0));
            pn.s1 = cfma(ar, self.s1, cscale(bt, pi.s1));
            st64(t64w, e, tn);
            st64(p64, e, pn);
            v[3 * r] += tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y +
                        S.shift[r] * (pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y);
          }
        } else {
          const M32 m[3] = {S.H32[i], S.H32[Ns + i], S.H32[2 * Ns + i]};
          const float dg = __ldg(S.diag32 + i);
          const int jj[3] = {j0, j1, j2};
#pragma unroll
          for (int r = 0; r < R; r++) {
            if (r >= nr || !sc.active[r]) continue;
            const int e = i * R + r;
            const Sp32 self = ld32(r32, e);
            Sp32 o{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
#pragma unroll
            for (int k = 0; k < 3; k++) {
              const Sp32 bk = LoField<P>::ld(rh, jj[k] * R + r);
              o.s0 = cfmaf(make_float2(m[k].r0.x, m[k].r0.y), bk.s0, o.s0);
              o.s0 = cfmaf(make_float2(m[k].r0.z, m[k].r0.w), bk.s1, o.s0);
              o.s1 = cfmaf(make_float2(m[k].r1.x, m[k].r1.y), bk.s0, o.s1);
              o.s1 = cfmaf(make_float2(m[k].r1.z, m[k].r1.w), bk.s1, o.s1);
            }
            const Sp32 ti = ld32(t32, e), pi = ld32(p32, e);
            const float2 ar = make_float2(float(sc.a_r[r].x), float(sc.a_r[r].y));
            const float bt = float(sc.beta[r]);
            Sp32 tn, pn;
            tn.s0 = cfmaf(ar, o.s0, make_float2(bt * ti.s0.x, bt * ti.s0.y));
            tn.s1 = cfmaf(ar, o.s1, make_float2(bt * ti.s1.x, bt * ti.s1.y));
            pn.s0 = cfmaf(ar, self.s0, make_float2(bt * pi.s0.x, bt * pi.s0.y));
            pn.s1 = cfmaf(ar, self.s1, make_float2(bt * pi.s1.x, bt * pi.s1.y));
            st32(t32, e, tn);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(th), e, tn);
            st32(p32, e, pn);
            const float tt = tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y;
            const float pp = pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y;
            vf[r] += tt + float(S.shift[r]) * pp;
          }
        }
      }
      if constexpr (mixed)
#pragma unroll
        for (int r = 0; r < R; r++) v[3 * r] += double(vf[r]);
    } else if (st == ST_B) {
      float vf[R];
#pragma unroll
      for (int r = 0; r < R; r++) vf[r] = 0.f;
      for (int i = tid; i < Ns; i += nth) {
        const int j0 = __ldg(S.nbr + i), j1 = __ldg(S.nbr + Ns + i), j2 = __ldg(S.nbr + 2 * Ns + i);
        if constexpr (!mixed) {
          const M64 m0 = S.Hd[i], m1 = S.Hd[Ns + i], m2 = S.Hd[2 * Ns + i];
          const double dg = __ldg(S.diag + i);
#pragma unroll
          for (int r = 0; r < R; r++) {
            if (r >= nr || !sc.active[r]) continue;
            const int e = i * R + r;
            const Sp64 self = ld64(t64w, e), b0 = ld64(t64w, j0 * R + r), b1 = ld64(t64w, j1 * R + r),
                       b2 = ld64(t64w, j2 * R + r);
            Sp64 q{cscale(dg, self.s0), cscale(dg, self.s1)};
            const M64* ms[3] = {&m0, &m1, &m2};
            const Sp64* bs[3] = {&b0, &b1, &b2};
#pragma unroll
            for (int k = 0; k < 3; k++) {
              q.s0 = cfma(ms[k]->h00, bs[k]->s0, q.s0);
              q.s0 = cfma(ms[k]->h01, bs[k]->s1, q.s0);
              q.s1 = cfma(ms[k]->h10, bs[k]->s0, q.s1);
              q.s1 = cfma(ms[k]->h11, bs[k]->s1, q.s1);
            }
            const Sp64 pi = ld64(p64, e), ri = ld64(r64, e), xi = ld64(xa, e);
            const double al = sc.alpha[r], s = S.shift[r];
            Sp64 rn, xn;
            rn.s0 = csub(ri.s0, cscale(al, cadd(q.s0, cscale(s, pi.s0))));
            rn.s1 = csub(ri.s1, cscale(al, cadd(q.s1, cscale(s, pi.s1))));
            xn.s0 = cadd(xi.s0, cscale(al, pi.s0));
            xn.s1 = cadd(xi.s1, cscale(al, pi.s1));
            st64(r64, e, rn);
            st64(xa, e, xn);
            v[3 * r] += rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y;
          }
        } else {
          const M32 m[3] = {S.Hd32[i], S.Hd32[Ns + i], S.Hd32[2 * Ns + i]};
          const float dg = __ldg(S.diag32 + i);
          const int jj[3] = {j0, j1, j2};
#pragma unroll
          for (int r = 0; r < R; r++) {
            if (r >= nr || !sc.active[r]) continue;
            const int e = i * R + r;
            const Sp32 self = ld32(t32, e);
            Sp32 q{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
#pragma unroll
            for (int k = 0; k < 3; k++) {
              const Sp32 bk = LoField<P>::ld(th, jj[k] * R + r);
              q.s0 = cfmaf(make_float2(m[k].r0.x, m[k].r0.y), bk.s0, q.s0);
              q.s0 = cfmaf(make_float2(m[k].r0.z, m[k].r0.w), bk.s1, q.s0);
              q.s1 = cfmaf(make_float2(m[k].r1.x, m[k].r1.y), bk.s0, q.s1);
              q.s1 = cfmaf(make_float2(m[k].r1.z, m[k].r1.w), bk.s1, q.s1);
            }
            const Sp32 pi = ld32(p32, e), ri = ld32(r32, e), xi = ld32(xlo, e);
            const float al = float(sc.alpha[r]), sf = float(S.shift[r]);
            Sp32 rn, xn;
            rn.s0 = make_float2(ri.s0.x - al * (q.s0.x + sf * pi.s0.x), ri.s0.y - al * (q.s0.y + sf * pi.s0.y));
            rn.s1 = make_float2(ri.s1.x - al * (q.s1.x + sf * pi.s1.x), ri.s1.y - al * (q.s1.y + sf * pi.s1.y));
            xn.s0 = make_float2(xi.s0.x + al * pi.s0.x, xi.s0.y + al * pi.s0.y);
            xn.s1 = make_float2(xi.s1.x + al * pi.s1.x, xi.s1.y + al * pi.s1.y);
            st32(r32, e, rn);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(rh), e, rn);
            st32(xlo, e, xn);
            vf[r] += rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y;
          }
        }
      }
      if constexpr (mixed)
#pragma unroll
        for (int r = 0; r < R; r++) v[3 * r] += double(vf[r]);
    } else if (st == ST_R1) {
      // t64 = D (x_hi + x_lo);  x_hi2 = x_hi + x_lo
      for (int i = tid; i < Ns; i += nth) {
        const int jj[3] = {__ldg(S.nbr + i), __ldg(S.nbr + Ns + i), __ldg(S.nbr + 2 * Ns + i)};
        const M64 m[3] = {S.H[i], S.H[Ns + i], S.H[2 * Ns + i]};
        const double dg = __ldg(S.diag + i);
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r >= nr) continue;
          if (!sc.active[r]) {
            // a finished right-hand side keeps its solution across the
            // buffer swap that follows this phase
            if constexpr (mixed) st64(xb, i * R + r, ld64(xa, i * R + r));
            continue;
          }
          auto xs = [&](int site) {
            const int e = site * R + r;
            const Sp64 h = ld64(xa, e);
            if constexpr (!mixed) {
              return h;
            } else {
              const Sp32 l = ld32(xlo, e);
              return Sp64{make_double2(h.s0.x + l.s0.x, h.s0.y + l.s0.y), make_double2(h.s1.x + l.s1.x, h.s1.y + l.s1.y)};
            }
          };
          const Sp64 self = xs(i);
          st64(xb, i * R + r, self);
          Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const Sp64 bj = xs(jj[k]);
            o.s0 = cfma(m[k].h00, bj.s0, o.s0);
            o.s0 = cfma(m[k].h01, bj.s1, o.s0);
            o.s1 = cfma(m[k].h10, bj.s0, o.s1);
            o.s1 = cfma(m[k].h11, bj.s1, o.s1);
          }
          st64(S.t64, i * R + r, o);
        }
      }
    } else if (st == ST_R2) {
      for (int i = tid; i < Ns; i += nth) {
        const int jj[3] = {__ldg(S.nbr + i), __ldg(S.nbr + Ns + i), __ldg(S.nbr + 2 * Ns + i)};
        const M64 m[3] = {S.Hd[i], S.Hd[Ns + i], S.Hd[2 * Ns + i]};
        const double dg = __ldg(S.diag + i);
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r >= nr || !sc.active[r]) continue;
          const int e = i * R + r;
          const Sp64 self = ld64(S.t64, e);
          Sp64 q{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const Sp64 bj = ld64(S.t64, jj[k] * R + r);
            q.s0 = cfma(m[k].h00, bj.s0, q.s0);
            q.s0 = cfma(m[k].h01, bj.s1, q.s0);
            q.s1 = cfma(m[k].h10, bj.s0, q.s1);
            q.s1 = cfma(m[k].h11, bj.s1, q.s1);
          }
          const Sp64 bi = ld64(S.b, e), xi = ld64(xa, e);
          const double s = S.shift[r];
          Sp64 rt;
          rt.s0 = csub(bi.s0, cadd(q.s0, cscale(s, xi.s0)));
          rt.s1 = csub(bi.s1, cadd(q.s1, cscale(s, xi.s1)));
          v[3 * r] += rt.s0.x * rt.s0.x + rt.s0.y * rt.s0.y + rt.s1.x * rt.s1.x + rt.s1.y * rt.s1.y;
          double2 pv0, pv1;
          if constexpr (!mixed) {
            const Sp64 pi = ld64(p64, e);
            pv0 = pi.s0;
            pv1 = pi.s1;
            st64(r64, e, rt);
          } else {
            const Sp32 pi = ld32(p32, e);
            pv0 = make_double2(pi.s0.x, pi.s0.y);
            pv1 = make_double2(pi.s1.x, pi.s1.y);
            const Sp32 rl{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
            st32(r32, e, rl);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(rh), e, rl);
            st32(xlo, e, Sp32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)});
          }
          v[3 * r + 1] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
          v[3 * r + 2] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
        }
      }
    }
    // ======================= publish + barrier =======================
    block_sum<3 * R>(v, sh);
    if (threadIdx.x == 0) {
      double* pp = part_ptr(a.partials, parity, R3);
#pragma unroll
      for (int q = 0; q < 3 * R; q++) __stcg(pp + q, v[q]);
    }
    int all_done = 0;
    if (!grid_sync_vote(a.bar, gen, a.spin_limit, st == ST_DONE, all_done)) {
      if (blockIdx.x == S.blk0 && threadIdx.x == 0) a.status[sidx] = QED3_ERR_TIMEOUT;
      return;
    }
    if (all_done) break;
    if (st == ST_DONE) {
      parity ^= 1;
      continue;
    }
    // ======================= system reduction =======================
    if (threadIdx.x < 32) {
      double acc[3 * R];
#pragma unroll
      for (int q = 0; q < 3 * R; q++) acc[q] = 0.0;
      for (int bI = S.blk0 + int(threadIdx.x); bI < S.blk1; bI += 32) {
        const double* pp = a.partials + (size_t(parity) * gridDim.x + bI) * R3;
#pragma unroll
        for (int q = 0; q < 3 * R; q++) acc[q] += __ldcg(pp + q);
      }
#pragma unroll
      for (int q = 0; q < 3 * R; q++) acc[q] = warp_sum(acc[q]);
      if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < 3 * R; q++) tot[q] = acc[q];
    }
    __syncthreads();
    parity ^= 1;
    // ======================= state transition (identical in all blocks of S) ==
    if (st == ST_INIT) {
      bool any = false;
      for (int r = 0; r < nr; r++) {
        sc.bnorm2[r] = tot[3 * r];
        sc.mu[r] = sc.mu_max[r] = sc.mu_true[r] = sc.bnorm2[r];
        if (sc.bnorm2[r] == 0.0) {
          sc.active[r] = 0;
          sc.status[r] = QED3_OK;
        } else {
          any = true;
        }
      }
      sc.state = any ? ST_A : ST_DONE;
    } else if (st == ST_A) {
      for (int r = 0; r < nr; r++)
        if (sc.active[r]) sc.alpha[r] = sc.mu[r] / tot[3 * r];
      sc.state = ST_B;
    } else if (st == ST_B) {
      sc.iter++;
      bool want = sc.iter >= a.maxiter;
      for (int r = 0; r < nr; r++) {
        if (!sc.active[r]) continue;
        const double mn = tot[3 * r];
        sc.mu_max[r] = fmax(sc.mu_max[r], mn);
        if (!isfinite(mn) || !isfinite(sc.alpha[r]) || mn < tol2 * sc.bnorm2[r] || (mixed && mn < delta2 * sc.mu_max[r]))
          want = true;
      }
      if (want) {
        // reliable update of every right-hand side of the system; mu keeps
        // the residual norm BEFORE this step for the next beta
        sc.state = ST_R1;
      } else {
        for (int r = 0; r < nr; r++) {
          if (!sc.active[r]) continue;
          const double mn = tot[3 * r];
          sc.beta[r] = mn / sc.mu[r];
          sc.a_r[r] = make_double2(1.0, 0.0);
          sc.mu[r] = mn;
        }
        sc.state = ST_A;
      }
    } else if (st == ST_R1) {
      if constexpr (mixed) {
        S64* tmp = xa;
        xa = xb;
        xb = tmp;
        sc.xsel ^= 1;
      }
      sc.state = ST_R2;
    } else if (st == ST_R2) {
      sc.nru++;
      bool any = false;
      for (int r = 0; r < nr; r++) {
        if (!sc.active[r]) continue;
        const double mt = tot[3 * r];
        sc.mu_true[r] = mt;
        if (mt < tol2 * sc.bnorm2[r]) {
          sc.active[r] = 0;
          sc.status[r] = QED3_OK;
          sc.it_done[r] = sc.iter;
          continue;
        }
        if (sc.iter >= a.maxiter || !isfinite(mt)) {
          sc.active[r] = 0;
          sc.status[r] = QED3_ERR_NOCONV;
          sc.it_done[r] = sc.iter;
          continue;
        }
        any = true;
        const double bt = mt / sc.mu[r];
        sc.beta[r] = bt;
        sc.a_r[r] = make_double2(1.0 - bt * tot[3 * r + 1] / mt, -bt * tot[3 * r + 2] / mt);
        sc.mu[r] = mt;
        sc.mu_max[r] = mt;
      }
      sc.state = any ? ST_A : ST_DONE;
    }
    if (sc.state == ST_DONE && blockIdx.x == S.blk0 && threadIdx.x == 0) {
      for (int r = 0; r < nr; r++) {
        double* o = S.scal + 6 * r;
        o[0] = sc.mu_true[r];
        o[1] = sc.bnorm2[r];
        o[2] = sc.it_done[r];
        o[3] = sc.nru;
        o[4] = sc.status[r];
        o[5] = sc.xsel;
      }
      a.status[sidx] = QED3_OK;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int P, int R>
static const void* batch_kernel(int threads) {
  return threads == 128 ? (const void*)k_batched_cg<P, R, 128> : (const void*)k_batched_cg<P, R, 256>;
}

template <int P, int R>
static int launch(BatchArgs& args, int grid, int threads, cudaStream_t st) {
  void* kargs[] = {&args};
  QED3_CUDA_TRY(cudaLaunchCooperativeKernel(batch_kernel<P, R>(threads), dim3(grid), dim3(threads), kargs, 0, st));
  return QED3_OK;
}

template <int P, int R>
static int occupancy(int threads, int* per_sm) {
  QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_kernel<P, R>(threads), threads, 0));
  return QED3_OK;
}

#define QED3_DISPATCH_R(P, R, fn, ...)                       \
  (R == 1 ? fn<P, 1>(__VA_ARGS__)                            \
   : R == 2 ? fn<P, 2>(__VA_ARGS__)                          \
   : R == 4 ? fn<P, 4>(__VA_ARGS__)                          \
            : fn<P, 8>(__VA_ARGS__))

int batch_occupancy(int prec, int R, int threads, int* per_sm) {
  if (prec == QED3_PREC_F64) return QED3_DISPATCH_R(P64, R, occupancy, threads, per_sm);
  if (prec == QED3_PREC_F32) return QED3_DISPATCH_R(P32, R, occupancy, threads, per_sm);
  return QED3_DISPATCH_R(PBF16, R, occupancy, threads, per_sm);
}

int batch_launch(int prec, int R, BatchArgs& args, int grid, int threads, cudaStream_t st) {
  if (prec == QED3_PREC_F64) return QED3_DISPATCH_R(P64, R, launch, args, grid, threads, st);
  if (prec == QED3_PREC_F32) return QED3_DISPATCH_R(P32, R, launch, args, grid, threads, st);
  return QED3_DISPATCH_R(PBF16, R, launch, args, grid, threads, st);
}

// Right-hand-side norms |b_r| (reference order, one block per right-hand
// side, fixed summation order).  The solve runs on b / |b| and the solution is
// scaled back on export, so the reduced-precision iterations see unit-scale
// vectors whatever the scale of b: an FP32 residual of a tiny right-hand side
// would otherwise underflow before the tolerance.
__global__ void k_rhs_norm(int Ns, int nrhs, long long stride, const S64* __restrict__ in, double* __restrict__ nrm) {
  __shared__ double sh[32];
  const int r = blockIdx.x;
  if (r >= nrhs) return;
  double v[1] = {0.0};
  for (int x = threadIdx.x; x < Ns; x += blockDim.x) {
    const Sp64 a = ld64(in + size_t(r) * stride, x);
    v[0] += a.s0.x * a.s0.x + a.s0.y * a.s0.y + a.s1.x * a.s1.x + a.s1.y * a.s1.y;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) nrm[r] = sqrt(v[0]);
}

// import nrhs reference-order vectors, each divided by its norm, into a
// site-major interleaved field
__global__ void k_import_interleaved(int Ns, int R, int nrhs, long long stride, const int* __restrict__ perm,
                                     const S64* __restrict__ in, const double* __restrict__ nrm,
                                     S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int x = perm[i];
  for (int r = 0; r < R; r++) {
    Sp64 v{make_double2(0, 0), make_double2(0, 0)};
    if (r < nrhs && nrm[r] > 0.0) {
      const double inv = 1.0 / nrm[r];
      v = ld64(in + size_t(r) * stride, x);
      v.s0 = cscale(inv, v.s0);
      v.s1 = cscale(inv, v.s1);
    }
    st64(out, i * R + r, v);
  }
}
__global__ void k_export_interleaved(int Ns, int R, int nrhs, const int* __restrict__ perm, const S64* __restrict__ in0,
                                     const S64* __restrict__ in1, const double* __restrict__ scal,
                                     const double* __restrict__ nrm, S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int x = perm[i];
  for (int r = 0; r < nrhs; r++) {
    const S64* src = (scal[6 * r + 5] != 0.0) ? in1 : in0;
    Sp64 v = ld64(src, i * R + r);
    v.s0 = cscale(nrm[r], v.s0);
    v.s1 = cscale(nrm[r], v.s1);
    st64(out + size_t(r) * Ns, x, v);
  }
}

int batch_import(const BatchSys& s, const qed3_dirac_s* d, const double* b_ref, int R, bool bcast, cudaStream_t st) {
  const long long stride = bcast ? 0LL : (long long)s.Ns;
  k_rhs_norm<<<s.nrhs, 256, 0, st>>>(s.Ns, s.nrhs, stride, reinterpret_cast<const S64*>(b_ref), s.bnorm);
  k_import_interleaved<<<(s.Ns + 255) / 256, 256, 0, st>>>(s.Ns, R, s.nrhs, stride, d->lat->dev.perm,
                                                         reinterpret_cast<const S64*>(b_ref), s.bnorm,
                                                         const_cast<S64*>(s.b));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int batch_export(const BatchSys& s, const qed3_dirac_s* d, double* x_ref, int R, cudaStream_t st) {
  k_export_interleaved<<<(s.Ns + 255) / 256, 256, 0, st>>>(s.Ns, R, s.nrhs, d->lat->dev.perm, s.xhi, s.xhi2, s.scal,
                                                         s.bnorm, reinterpret_cast<S64*>(x_ref));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

}  // namespace qed3

// ===========================================================================
// Batch handle: creation (block partition, workspaces), solve, autotuner
// ===========================================================================
namespace qed3 {

// Dynamic-schedule counters in one int buffer: tiles done [nsys], steps
// completed [nsys], the 64-bit work counter (8-byte aligned), systems done.
static int dyn_work_offset(int nsys) { return (2 * nsys + 1) & ~1; }
static int dyn_counter_ints(int nsys) { return dyn_work_offset(nsys) + 4; }

static void batch_release(qed3_batch_s* bt) {
  for (void* p : bt->buffers)
    if (p) cudaFree(p);
  bt->buffers.clear();
  void* ptrs[] = {bt->d_sys,         bt->d_sys_of_block, bt->partials, bt->bar,        bt->d_status,
                  bt->d_scal,        bt->d_sys_of_tile,  bt->d_dyn,    bt->d_counters, bt->d_tile_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  bt->d_sys_of_tile = nullptr;
  bt->d_dyn = nullptr;
  bt->d_counters = nullptr;
  bt->d_tile_part = nullptr;
  bt->d_sys = nullptr;
  bt->d_sys_of_block = nullptr;
  bt->partials = nullptr;
  bt->bar = nullptr;
  bt->d_status = nullptr;
  bt->d_scal = nullptr;
  if (bt->e0) cudaEventDestroy(bt->e0);
  if (bt->e1) cudaEventDestroy(bt->e1);
  bt->e0 = bt->e1 = nullptr;
}

// Splits the launch's blocks over the internal systems in proportion to their
// expected work: sites x right-hand sides x iterations per right-hand side,
// the last taken from the previous synchronous solve (1 before the first).
// All systems advance through the same grid barriers, so a system that needs
// twice the iterations of the others gets twice their blocks per site and
// finishes with them instead of running on alone.  At least one block per
// system and no more blocks than site slots (T sites per block pass).  The total is fixed when the batch is built, so a launch
// captured in a CUDA graph stays valid after a re-split: only the contents of
// the block-to-system table and the descriptors change.
static void batch_partition(qed3_batch_s* bt) {
  const int nsys = int(bt->sys.size());
  const int slots = bt->threads;
  std::vector<long long> maxb(nsys);
  long long room = 0;
  for (int i = 0; i < nsys; i++) {
    maxb[i] = (bt->sys[i].Ns + slots - 1) / slots;
    room += maxb[i];
  }
  if (bt->grid <= 0) bt->grid = int(std::min(bt->cap, room));
  const long long G = bt->grid;
  double wsum = 0;
  for (int i = 0; i < nsys; i++) wsum += double(bt->sys[i].Ns) * bt->sys[i].nrhs * bt->work[i];
  std::vector<double> ideal(nsys);
  std::vector<long long> nb(nsys);
  long long tot = 0;
  for (int i = 0; i < nsys; i++) {
    const BatchSys& s = bt->sys[i];
    ideal[i] = double(G) * double(s.Ns) * s.nrhs * bt->work[i] / wsum;
    nb[i] = std::max(1LL, std::min((long long)std::floor(ideal[i]), maxb[i]));
    tot += nb[i];
  }
  while (tot > G) {  // trim the allocation furthest above its share
    int imax = -1;
    for (int i = 0; i < nsys; i++)
      if (nb[i] > 1 && (imax < 0 || nb[i] - ideal[i] > nb[imax] - ideal[imax])) imax = i;
    if (imax < 0) break;
    nb[imax]--;
    tot--;
  }
  while (tot < G) {  // hand out the rest to the allocation furthest below its share
    int imin = -1;
    for (int i = 0; i < nsys; i++)
      if (nb[i] < maxb[i] && (imin < 0 || nb[i] - ideal[i] < nb[imin] - ideal[imin])) imin = i;
    if (imin < 0) break;
    nb[imin]++;
    tot++;
  }
  bt->sob.clear();
  for (int i = 0; i < nsys; i++) {
    bt->sys[i].blk0 = int(bt->sob.size());
    for (long long k = 0; k < nb[i]; k++) bt->sob.push_back(i);
    bt->sys[i].blk1 = int(bt->sob.size());
  }
}

// Re-splits the blocks from the iteration counts of the solve just reported
// (the scalars already copied to the host) and uploads the new table and
// descriptors on st.  Called only from the synchronous solve, never while a
// stream is being captured.
static int batch_rebalance(qed3_batch_s* bt, const std::vector<double>& scal, cudaStream_t st) {
  const int R = bt->R, nsys = int(bt->sys.size());
  std::vector<double> w(nsys);
  for (int i = 0; i < nsys; i++) {
    double s = 0;
    for (int r = 0; r < bt->sys[i].nrhs; r++) s += scal[size_t(6) * R * i + 6 * r + 2];
    w[i] = 1.0 + s / bt->sys[i].nrhs;
  }
  const std::vector<int> old = bt->sob;
  bt->work = w;
  batch_partition(bt);
  if (bt->sob == old) return QED3_OK;
  QED3_CUDA_TRY(cudaMemcpyAsync(bt->d_sys_of_block, bt->sob.data(), sizeof(int) * bt->sob.size(),
                                cudaMemcpyHostToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(bt->d_sys, bt->sys.data(), sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice, st));
  return QED3_OK;
}

static int batch_build(qed3_batch_s* bt) {
  const int R = bt->R;
  bt->sys_uploaded = false;
  bt->sys.clear();
  bt->owner.clear();
  bt->first_rhs.clear();
  for (size_t u = 0; u < bt->user_ops.size(); u++) {
    qed3_dirac_s* d = bt->user_ops[u];
    if (!d->coeffs_set) return fail(QED3_ERR_STATE, "batch operator without coefficients");
    for (int f = 0; f < bt->user_nrhs[u]; f += R) {
      BatchSys s{};
      s.Ns = d->Ns;
      s.nrhs = std::min(R, bt->user_nrhs[u] - f);
      s.nbr = d->lat->dev.nbr;
      s.H = d->H;
      s.Hd = d->Hd;
      s.diag = d->diag;
      s.H32 = d->H32;
      s.Hd32 = d->Hd32;
      s.diag32 = d->diag32;
      bt->sys.push_back(s);
      bt->owner.push_back(int(u));
      bt->first_rhs.push_back(f);
    }
  }
  const int nsys = int(bt->sys.size());
  const bool dyn = bt->sched == QED3_BATCH_DYNAMIC;
  int dev = 0, smc = 0, per_sm = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  QED3_CUDA_TRY(cudaDeviceGetAttribute(&smc, cudaDevAttrMultiProcessorCount, dev));
  int rc = dyn ? batch_dyn_occupancy(bt->prec, R, bt->threads, &per_sm) : batch_occupancy(bt->prec, R, bt->threads, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return fail(QED3_ERR_CUDA, "batched CG kernel cannot be resident");
  bt->cap = (long long)per_sm * smc;
  std::vector<int> sot;
  if (dyn) {
    // warp tiles of 32 x spt consecutive sites, system after system: about
    // eight tiles per co-resident warp and step while every system is active,
    // but at least 8 sites per thread (below that the tile's counter, state
    // reads and sums cost more than the balance gains; measured on the
    // 256-RHS batch: 3 sites per thread 211 ms, 7: 159 ms, 15: 164 ms)
    double work = 0;  // site x right-hand-side pairs
    for (const auto& s : bt->sys) work += double(s.Ns) * s.nrhs;
    bt->spt = int(std::max(8.0, std::min(32.0, std::floor(work / (8.0 * bt->cap * bt->threads * bt->R)))));
    const int tile = 32 * bt->spt;
    for (int i = 0; i < nsys; i++) {
      BatchSys& s = bt->sys[i];
      s.ch0 = int(sot.size());
      for (int c = 0; c < (s.Ns + tile - 1) / tile; c++) sot.push_back(i);
      s.ch1 = int(sot.size());
      s.blk0 = s.blk1 = 0;
    }
    bt->ntiles = int(sot.size());
    bt->grid = int(bt->cap);
  } else {
    if (bt->cap < nsys) return fail(QED3_ERR_ARG, "more systems than co-resident blocks; use a larger right-hand-side tile");
    bt->work.assign(nsys, 1.0);
    bt->grid = 0;
    batch_partition(bt);
  }
  // workspaces
  for (auto& s : bt->sys) {
    const size_t bytes = size_t(s.Ns) * R * sizeof(S64);
    void* p[10];
    for (int k = 0; k < 10; k++) {
      QED3_CUDA_TRY(cudaMalloc(&p[k], bytes));
      bt->buffers.push_back(p[k]);
    }
    s.b = reinterpret_cast<S64*>(p[0]);
    s.xhi = reinterpret_cast<S64*>(p[1]);
    s.xhi2 = reinterpret_cast<S64*>(p[2]);
    s.t64 = reinterpret_cast<S64*>(p[3]);
    s.r = p[4];
    s.p = p[5];
    s.t = p[6];
    s.xlo = p[7];
    s.rh = p[8];
    s.th = p[9];
  }
  QED3_CUDA_TRY(cudaMalloc(&bt->d_scal, sizeof(double) * 7 * R * nsys));
  for (int i = 0; i < nsys; i++) {
    bt->sys[i].scal = bt->d_scal + size_t(6) * R * i;
    bt->sys[i].bnorm = bt->d_scal + size_t(6) * R * nsys + size_t(R) * i;
  }
  QED3_CUDA_TRY(cudaMalloc(&bt->d_sys, sizeof(BatchSys) * nsys));
  if (dyn) {
    QED3_CUDA_TRY(cudaMalloc(&bt->d_sys_of_tile, sizeof(int) * sot.size()));
    QED3_CUDA_TRY(cudaMemcpy(bt->d_sys_of_tile, sot.data(), sizeof(int) * sot.size(), cudaMemcpyHostToDevice));
    QED3_CUDA_TRY(cudaMalloc(&bt->d_dyn, sizeof(DynState<kMaxTile>) * nsys));
    QED3_CUDA_TRY(cudaMalloc(&bt->d_counters, sizeof(int) * dyn_counter_ints(nsys)));
    QED3_CUDA_TRY(cudaMalloc(&bt->d_tile_part, sizeof(double) * 3 * R * sot.size()));
  } else {
    QED3_CUDA_TRY(cudaMalloc(&bt->d_sys_of_block, sizeof(int) * bt->cap));
    QED3_CUDA_TRY(cudaMemcpy(bt->d_sys_of_block, bt->sob.data(), sizeof(int) * bt->sob.size(), cudaMemcpyHostToDevice));
    QED3_CUDA_TRY(cudaMalloc(&bt->partials, sizeof(double) * 2 * bt->cap * 3 * R));
  }
  QED3_CUDA_TRY(cudaMalloc(&bt->bar, sizeof(GridBar)));
  QED3_CUDA_TRY(cudaMalloc(&bt->d_status, sizeof(int) * nsys));
  QED3_CUDA_TRY(cudaEventCreate(&bt->e0));
  QED3_CUDA_TRY(cudaEventCreate(&bt->e1));
  return QED3_OK;
}

// Writes the per-right-hand-side shifts into the device descriptors.  The copy
// is made only when a shift changed since the last upload, from pageable host
// memory (staged by the runtime before the call returns), so it is never part
// of a captured launch sequence.
int batch_set_shifts(qed3_batch_s* bt, const double* const* shifts, double shift, cudaStream_t st) {
  const int nsys = int(bt->sys.size());
  bool changed = !bt->sys_uploaded;
  for (int i = 0; i < nsys; i++) {
    BatchSys& s = bt->sys[i];
    const int u = bt->owner[i], f = bt->first_rhs[i];
    for (int r = 0; r < kMaxTile; r++) {
      const double v = r < s.nrhs ? ((shifts && shifts[u]) ? shifts[u][f + r] : shift) : 0.0;
      if (v != s.shift[r]) changed = true;
      s.shift[r] = v;
    }
  }
  if (!changed) return QED3_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  QED3_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone)
    return fail(QED3_ERR_STATE, "batch shifts changed during stream capture; set them before capturing");
  QED3_CUDA_TRY(cudaMemcpyAsync(bt->d_sys, bt->sys.data(), sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice, st));
  bt->sys_uploaded = true;
  return QED3_OK;
}

// Enqueues one batched solve on st: gather of the right-hand sides, the
// persistent cooperative launch and the scatter of the solutions.  No host
// synchronisation, allocation or host-to-device copy: the sequence can be
// captured into a CUDA graph and replayed (the graph keeps x, b and the
// shifts set before capture).
int batch_launch_all(qed3_batch_s* bt, double* const* x, const double* const* b, const qed3_solve_params* prm,
                     cudaStream_t st) {
  if (!bt->sys_uploaded) return fail(QED3_ERR_STATE, "batch shifts not set");
  const int R = bt->R, nsys = int(bt->sys.size());
  const bool bcast = prm && (prm->flags & QED3_SOLVE_BCAST_B);
  for (int i = 0; i < nsys; i++) {
    const BatchSys& s = bt->sys[i];
    const int u = bt->owner[i], f = bt->first_rhs[i];
    const int rc = batch_import(s, bt->user_ops[u], bcast ? b[u] : b[u] + size_t(f) * 4 * s.Ns, R, bcast, st);
    if (rc) return rc;
  }
  QED3_CUDA_TRY(cudaMemsetAsync(bt->bar, 0, sizeof(GridBar), st));
  QED3_CUDA_TRY(cudaMemsetAsync(bt->d_status, 0xff, sizeof(int) * nsys, st));
  const double tol = prm && prm->tol > 0 ? prm->tol : 1e-10;
  const double delta = prm && prm->delta > 0 ? prm->delta : 0.1;
  const int maxiter = prm && prm->maxiter > 0 ? prm->maxiter : 100000;
  int rc = QED3_OK;
  if (bt->sched == QED3_BATCH_DYNAMIC) {
    QED3_CUDA_TRY(cudaMemsetAsync(bt->d_dyn, 0, sizeof(DynState<kMaxTile>) * nsys, st));
    QED3_CUDA_TRY(cudaMemsetAsync(bt->d_counters, 0, sizeof(int) * dyn_counter_ints(nsys), st));
    DynArgs a{};
    a.sys = bt->d_sys;
    a.nsys = nsys;
    a.sys_of_tile = bt->d_sys_of_tile;
    a.ntiles = bt->ntiles;
    a.spt = bt->spt;
    a.state = bt->d_dyn;
    a.sys_cnt = bt->d_counters;
    a.epoch = bt->d_counters + nsys;
    a.work = reinterpret_cast<unsigned long long*>(bt->d_counters + dyn_work_offset(nsys));
    a.ndone = bt->d_counters + dyn_work_offset(nsys) + 2;
    a.part = bt->d_tile_part;
    a.bar = bt->bar;
    a.status = bt->d_status;
    a.tol2 = tol * tol;
    a.delta2 = delta * delta;
    a.maxiter = maxiter;
    a.spin_limit = 20000000LL;
    if (bt->timing) QED3_CUDA_TRY(cudaEventRecord(bt->e0, st));
    rc = batch_dyn_launch(bt->prec, R, a, bt->grid, bt->threads, st);
  } else {
    BatchArgs a{};
    a.sys = bt->d_sys;
    a.sys_of_block = bt->d_sys_of_block;
    a.nsys = nsys;
    a.partials = bt->partials;
    a.bar = bt->bar;
    a.status = bt->d_status;
    a.tol2 = tol * tol;
    a.delta2 = delta * delta;
    a.maxiter = maxiter;
    a.spin_limit = 20000000LL;
    if (bt->timing) QED3_CUDA_TRY(cudaEventRecord(bt->e0, st));
    rc = batch_launch(bt->prec, R, a, bt->grid, bt->threads, st);
  }
  if (rc) return rc;
  if (bt->timing) QED3_CUDA_TRY(cudaEventRecord(bt->e1, st));
  for (int i = 0; i < nsys; i++) {
    const BatchSys& s = bt->sys[i];
    const int u = bt->owner[i], f = bt->first_rhs[i];
    if ((rc = batch_export(s, bt->user_ops[u], x[u] + size_t(f) * 4 * s.Ns, R, st))) return rc;
  }
  return QED3_OK;
}

// Waits for st and turns the device-side results of the last launch into
// reports (user order: system u, right-hand side j -> offset(u) + j).
int batch_reports(qed3_batch_s* bt, qed3_solve_report* reports, float ms, cudaStream_t st) {
  const int R = bt->R, nsys = int(bt->sys.size());
  std::vector<double> scal(size_t(6) * R * nsys);
  std::vector<int> status(nsys);
  QED3_CUDA_TRY(cudaMemcpyAsync(scal.data(), bt->d_scal, scal.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(status.data(), bt->d_status, status.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  bool timeout = false, missing = false;
  std::vector<int> off(bt->user_ops.size() + 1, 0);
  for (size_t u = 0; u < bt->user_ops.size(); u++) off[u + 1] = off[u] + bt->user_nrhs[u];
  for (int i = 0; i < nsys; i++) {
    if (status[i] == QED3_ERR_TIMEOUT) timeout = true;
    if (status[i] == -1) missing = true;  // still the launch's 0xff fill: the kernel never finished the system
    const BatchSys& s = bt->sys[i];
    for (int r = 0; r < s.nrhs; r++) {
      const double* o = &scal[size_t(6) * R * i + 6 * r];
      qed3_solve_report rep{};
      rep.status = status[i] == QED3_ERR_TIMEOUT ? QED3_ERR_TIMEOUT : int(o[4]);
      rep.iters = int(o[2]);
      rep.reliable_updates = int(o[3]);
      rep.true_rel_res = o[1] > 0 ? std::sqrt(o[0] / o[1]) : 0.0;
      rep.ms = ms;
      if (reports) reports[off[bt->owner[i]] + bt->first_rhs[i] + r] = rep;
    }
  }
  if (timeout) return fail(QED3_ERR_TIMEOUT, "grid barrier timed out inside the batched CG kernel");
  if (missing) return fail(QED3_ERR_STATE, "no completed batched launch to report on");
  bt->last_scal.swap(scal);
  return QED3_OK;
}

int batch_solve(qed3_batch_s* bt, double* const* x, const double* const* b, const double* const* shifts,
                const qed3_solve_params* prm, qed3_solve_report* reports, float* ms_out, cudaStream_t st) {
  int rc = batch_set_shifts(bt, shifts, prm ? prm->shift : 0.0, st);
  if (rc) return rc;
  bt->timing = true;
  rc = batch_launch_all(bt, x, b, prm, st);
  bt->timing = false;
  if (rc) return rc;
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  float ms = 0.f;
  QED3_CUDA_TRY(cudaEventElapsedTime(&ms, bt->e0, bt->e1));
  if (ms_out) *ms_out = ms;
  rc = batch_reports(bt, reports, ms, st);
  if (rc) return rc;
  return bt->sched == QED3_BATCH_DYNAMIC ? QED3_OK : batch_rebalance(bt, bt->last_scal, st);
}

// ---- autotuner ----------------------------------------------------------------
// Times a short solve (24 iterations, synthetic right-hand sides) for each
// (rhs tile, threads per block) candidate and keeps the fastest per
// (lattice sizes, right-hand-side counts, precision).  Results are cached for
// the life of the process.
struct TuneKey {
  std::vector<long long> sig;
  bool operator<(const TuneKey& o) const { return sig < o.sig; }
};
struct TuneBest {
  int R, T, sched;
};
static std::map<TuneKey, TuneBest>& tune_cache() {
  static std::map<TuneKey, TuneBest> c;
  return c;
}

__global__ void k_fill_synthetic(int n, double* v, unsigned seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned h = (unsigned(i) + 1u) * 2654435761u ^ seed * 40503u;
  h ^= h >> 15;
  h *= 2246822519u;
  h ^= h >> 13;
  v[i] = double(h & 0xffffff) / double(0x1000000) - 0.5;
}

int batch_autotune(qed3_batch_s* proto, int* best_R, int* best_threads, int* best_sched, std::vector<BatchTrial>* log) {
  TuneKey key;
  key.sig.push_back(proto->prec);
  key.sig.push_back(proto->R);
  key.sig.push_back(proto->threads);
  key.sig.push_back(proto->sched);
  int maxn = 1;
  for (size_t u = 0; u < proto->user_ops.size(); u++) {
    key.sig.push_back(proto->user_ops[u]->Ns);
    key.sig.push_back(proto->user_nrhs[u]);
    maxn = std::max(maxn, proto->user_nrhs[u]);
  }
  auto it = tune_cache().find(key);
  if (it != tune_cache().end() && !log) {
    *best_R = it->second.R;
    *best_threads = it->second.T;
    *best_sched = it->second.sched;
    return QED3_OK;
  }
  // synthetic right-hand sides
  std::vector<double*> xs, bs;
  for (size_t u = 0; u < proto->user_ops.size(); u++) {
    const size_t n = size_t(4) * proto->user_ops[u]->Ns * proto->user_nrhs[u];
    double *xb, *bb;
    QED3_CUDA_TRY(cudaMalloc(&xb, n * sizeof(double)));
    QED3_CUDA_TRY(cudaMalloc(&bb, n * sizeof(double)));
    k_fill_synthetic<<<int((n + 255) / 256), 256>>>(int(n), bb, unsigned(u + 1));
    xs.push_back(xb);
    bs.push_back(bb);
  }
  float best = 1e30f;
  int bR = 1, bT = 256, bS = QED3_BATCH_STATIC;
  qed3_solve_params p{1e-30, 24, proto->prec, 0.1, 0.0, 0};
  for (int sched : {QED3_BATCH_STATIC, QED3_BATCH_DYNAMIC}) {
    if (proto->sched > 0 && sched != proto->sched) continue;
    for (int R : {1, 2, 4, 8}) {
      if (R > 1 && R / 2 >= maxn) break;
      if (proto->R > 0 && R != proto->R) continue;
      for (int T : {128, 256}) {
        if (proto->threads > 0 && T != proto->threads) continue;
        qed3_batch_s trial;
        trial.prec = proto->prec;
        trial.R = R;
        trial.threads = T;
        trial.sched = sched;
        trial.user_ops = proto->user_ops;
        trial.user_nrhs = proto->user_nrhs;
        int rc = batch_build(&trial);
        float ms = 1e30f;
        if (rc == QED3_OK) {
          float m0 = 0.f, m1 = 0.f;
          rc = batch_solve(&trial, xs.data(), bs.data(), nullptr, &p, nullptr, &m0, 0);
          if (rc == QED3_OK || rc == QED3_ERR_NOCONV)
            rc = batch_solve(&trial, xs.data(), bs.data(), nullptr, &p, nullptr, &m1, 0);
          if (rc == QED3_OK || rc == QED3_ERR_NOCONV) ms = m1;
        }
        batch_release(&trial);
        if (log) log->push_back({R, T, sched, ms});
        if (ms < best) {
          best = ms;
          bR = R;
          bT = T;
          bS = sched;
        }
      }
    }
  }
  for (double* p2 : xs) cudaFree(p2);
  for (double* p2 : bs) cudaFree(p2);
  set_error("");
  if (best >= 1e29f) return fail(QED3_ERR_CUDA, "autotuner found no runnable configuration");
  tune_cache()[key] = {bR, bT, bS};
  *best_R = bR;
  *best_threads = bT;
  *best_sched = bS;
  return QED3_OK;
}

int batch_create(int nsys, qed3_dirac_s* const* ops, const int* nrhs, int prec, int rhs_tile, int threads,
                 qed3_batch_s** out, int sched) {
  auto* bt = new qed3_batch_s;
  bt->prec = prec;
  for (int u = 0; u < nsys; u++) {
    bt->user_ops.push_back(ops[u]);
    bt->user_nrhs.push_back(nrhs[u]);
  }
  int R = rhs_tile, T = threads, S = sched;
  if (S != 0 && S != QED3_BATCH_STATIC && S != QED3_BATCH_DYNAMIC) {
    delete bt;
    return fail(QED3_ERR_ARG, "schedule must be 0, QED3_BATCH_STATIC or QED3_BATCH_DYNAMIC");
  }
  if (R <= 0 || T <= 0) {
    // the autotuner picks what was left open (the schedule too, when 0)
    int aR = 1, aT = 256, aS = QED3_BATCH_STATIC;
    bt->R = R;
    bt->threads = T;
    bt->sched = S;
    const int rc = batch_autotune(bt, &aR, &aT, &aS, nullptr);
    if (rc) {
      delete bt;
      return rc;
    }
    if (R <= 0) R = aR;
    if (T <= 0) T = aT;
    if (S <= 0) S = aS;
  }
  if (S <= 0) S = QED3_BATCH_STATIC;
  if (!(R == 1 || R == 2 || R == 4 || R == 8)) {
    delete bt;
    return fail(QED3_ERR_ARG, "rhs_tile must be 1, 2, 4 or 8");
  }
  if (T != 128 && T != 256) {
    delete bt;
    return fail(QED3_ERR_ARG, "threads must be 128 or 256");
  }
  bt->R = R;
  bt->threads = T;
  bt->sched = S;
  const int rc = batch_build(bt);
  if (rc) {
    batch_release(bt);
    delete bt;
    return rc;
  }
  *out = bt;
  return QED3_OK;
}

void batch_destroy(qed3_batch_s* bt) {
  if (!bt) return;
  batch_release(bt);
  delete bt;
}

}  // namespace qed3
