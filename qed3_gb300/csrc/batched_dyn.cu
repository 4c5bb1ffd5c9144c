// Batched CG, dynamic schedule: the systems of a batch (see batched.cu) run the
// same per-system CG state machine
//     INIT -> (A -> B)* -> [R1 -> R2] -> ... -> DONE
// but no block is tied to a system and no grid barrier separates the steps.
// Every system is cut into warp tiles of 32 x spt consecutive sites (all R
// right-hand sides of a site together, so a tile reads each hop block once for
// R spinors).  A work item is one step of one tile, numbered
// step * ntiles + tile, and each warp takes items in increasing order from one
// counter (prefetching the next while it works).  A step of a system only
// depends on that system's previous step, so before working on an item the
// warp waits until its system has completed the previous step (a per-system
// epoch, release/acquire); systems in different steps overlap freely.  The
// warp publishes the tile's partial sums in the tile's own slot; the warp that
// completes a system's last tile of a step sums the slots in a fixed order,
// advances the system's state (in device memory) and releases the next step.
// Tiles of finished systems are skipped; every warp leaves when all systems
// are done.
//
// No deadlock: items are taken in order, so every item of step k was taken
// before any of step k + 1, and the lowest step held by any warp can always
// proceed.  Against the static schedule (each system owns a fixed range of
// blocks for the whole solve) the whole GPU works on whatever systems are
// still running, and a slow tile delays only its own system.  Sums are over
// fixed tile slots in a fixed order, so results do not depend on which warp
// took which tile: a replay gives bit-identical iterates.
//
// Counters and states are zeroed before each launch (stream-ordered memsets),
// and every wait is bounded: on expiry the warp sets the abort flag, every
// warp leaves, and the unfinished systems report a timeout.

#include <cuda_runtime.h>

#include "batched_impl.h"
#include "device.cuh"
#include "handles.h"

namespace qed3 {

namespace {

enum DynPhase { D_INIT = 0, D_A = 1, D_B = 2, D_R1 = 3, D_R2 = 4, D_DONE = 5 };

// The state transition of one system after a step, from its totals
// tot[3 r + q] (q = 0: the phase's squared norm, 1/2: Re/Im <r, p> after a
// reliable update).  Run by one thread; the state is read and written through
// volatile accesses (other blocks wrote it in earlier steps).
template <int R>
__device__ __noinline__ void dyn_transition(const DynArgs& a, const BatchSys& S, int sidx, volatile DynState<R>* d,
                               const double* tot, bool mixed, int* ndone) {
  const int nr = S.nrhs;
  const int st = d->state;
  int next = st;
  if (st == D_INIT) {
    bool any = false;
    for (int r = 0; r < R; r++) {
      if (r >= nr) {
        d->active[r] = 0;
        continue;
      }
      const double b2 = tot[3 * r];
      d->bnorm2[r] = b2;
      d->mu[r] = b2;
      d->mu_max[r] = b2;
      d->mu_true[r] = b2;
      d->beta[r] = 0.0;
      d->a_r[r].x = 1.0;
      d->a_r[r].y = 0.0;
      d->it_done[r] = 0;
      if (b2 == 0.0) {
        d->active[r] = 0;
        d->status[r] = QED3_OK;
      } else {
        d->active[r] = 1;
        d->status[r] = QED3_ERR_NOCONV;
        any = true;
      }
    }
    next = any ? D_A : D_DONE;
  } else if (st == D_A) {
    for (int r = 0; r < nr; r++)
      if (d->active[r]) d->alpha[r] = d->mu[r] / tot[3 * r];
    next = D_B;
  } else if (st == D_B) {
    const int iter = d->iter + 1;
    d->iter = iter;
    bool want = iter >= a.maxiter;
    for (int r = 0; r < nr; r++) {
      if (!d->active[r]) continue;
      const double mn = tot[3 * r];
      const double mx = fmax(d->mu_max[r], mn);
      d->mu_max[r] = mx;
      if (!isfinite(mn) || !isfinite(d->alpha[r]) || mn < a.tol2 * d->bnorm2[r] || (mixed && mn < a.delta2 * mx))
        want = true;
    }
    if (want) {
      next = D_R1;  // reliable update of every right-hand side; mu keeps the norm before this step
    } else {
      for (int r = 0; r < nr; r++) {
        if (!d->active[r]) continue;
        const double mn = tot[3 * r];
        d->beta[r] = mn / d->mu[r];
        d->a_r[r].x = 1.0;
        d->a_r[r].y = 0.0;
        d->mu[r] = mn;
      }
      next = D_A;
    }
  } else if (st == D_R1) {
    if (mixed) d->xsel = d->xsel ^ 1;
    next = D_R2;
  } else if (st == D_R2) {
    d->nru = d->nru + 1;
    const int iter = d->iter;
    bool any = false;
    for (int r = 0; r < nr; r++) {
      if (!d->active[r]) continue;
      const double mt = tot[3 * r];
      d->mu_true[r] = mt;
      if (mt < a.tol2 * d->bnorm2[r]) {
        d->active[r] = 0;
        d->status[r] = QED3_OK;
        d->it_done[r] = iter;
        continue;
      }
      if (iter >= a.maxiter || !isfinite(mt)) {
        d->active[r] = 0;
        d->status[r] = QED3_ERR_NOCONV;
        d->it_done[r] = iter;
        continue;
      }
      any = true;
      const double bt = mt / d->mu[r];
      d->beta[r] = bt;
      d->a_r[r].x = 1.0 - bt * tot[3 * r + 1] / mt;
      d->a_r[r].y = -bt * tot[3 * r + 2] / mt;
      d->mu[r] = mt;
      d->mu_max[r] = mt;
    }
    next = any ? D_A : D_DONE;
  }
  d->state = next;
  if (next == D_DONE) {
    for (int r = 0; r < nr; r++) {
      double* o = S.scal + 6 * r;
      o[0] = d->mu_true[r];
      o[1] = d->bnorm2[r];
      o[2] = d->it_done[r];
      o[3] = d->nru;
      o[4] = d->status[r];
      o[5] = d->xsel;
    }
    a.status[sidx] = QED3_OK;
    __threadfence();
    atomicAdd(ndone, 1);
  }
}

// ---- the work of one tile in each phase ----------------------------------------
// A tile is T x spt consecutive sites i0 + si * T (si < spt) of one system;
// each thread accumulates its sites' contributions to the system's sums in v.
// Each phase has its own loop so that only its own pointers and loads are
// live.  The FP64 phases (INIT, R1, R2) run a few times per solve; their
// neighbour loops are not unrolled, which keeps their register needs below
// those of A and B.
template <int P>
struct LoPtr {
  using T = typename LoField<P == P64 ? P32 : P>::T;
};

// The descriptor fields a tile loop uses, copied to registers before the loop
// (read through the descriptor, they would be reloaded after every store).
template <int R>
struct TileView {
  int Ns, nr;
  const int* __restrict__ nbr;
  double shift[R];
  __device__ explicit TileView(const BatchSys& S) : Ns(S.Ns), nr(S.nrhs), nbr(S.nbr) {
#pragma unroll
    for (int r = 0; r < R; r++) shift[r] = S.shift[r];
  }
};

// A: t = a_r D r + beta t,  p = a_r r + beta p;  v = |t|^2 + shift |p|^2
template <int P, int R, int T>
__device__ __forceinline__ void tile_A(const BatchSys& S, int i0, int spt, const int* __restrict__ act,
                                       const double* __restrict__ beta, const double* __restrict__ arx,
                                       const double* __restrict__ ary, double* v) {
  constexpr bool mixed = (P != P64);
  const TileView<R> V(S);
  const int Ns = V.Ns, nr = V.nr;
  if constexpr (!mixed) {
    const S64* __restrict__ r64 = reinterpret_cast<const S64*>(S.r);
    S64* __restrict__ p64 = reinterpret_cast<S64*>(S.p);
    S64* __restrict__ t64w = reinterpret_cast<S64*>(S.t);
    const M64* __restrict__ H = S.H;
    const double* __restrict__ diag = S.diag;
#pragma unroll 1
    for (int si = 0; si < spt; si++) {
      const int i = i0 + si * T;
      if (i >= Ns) break;
      const int jj[3] = {__ldg(V.nbr + i), __ldg(V.nbr + Ns + i), __ldg(V.nbr + 2 * Ns + i)};
      const M64 m[3] = {H[i], H[Ns + i], H[2 * Ns + i]};
      const double dg = __ldg(diag + i);
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (r >= nr || !act[r]) continue;
        const int e = i * R + r;
        const Sp64 self = ld64(r64, e);
        Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
        for (int k3 = 0; k3 < 3; k3++) {
          const Sp64 bk = ld64(r64, jj[k3] * R + r);
          o.s0 = cfma(m[k3].h00, bk.s0, o.s0);
          o.s0 = cfma(m[k3].h01, bk.s1, o.s0);
          o.s1 = cfma(m[k3].h10, bk.s0, o.s1);
          o.s1 = cfma(m[k3].h11, bk.s1, o.s1);
        }
        const Sp64 ti = ld64(t64w, e), pi = ld64(p64, e);
        const double bt = beta[r];
        const double2 ar = make_double2(arx[r], ary[r]);
        Sp64 tn, pn;
        tn.s0 = cfma(ar, o.s0, cscale(bt, ti.s0));
        tn.s1 = cfma(ar, o.s1, cscale(bt, ti.s1));
        pn.s0 = cfma(ar, self.s0, cscale(bt, pi.s0));
        pn.s1 = cfma(ar, self.s1, cscale(bt, pi.s1));
        st64(t64w, e, tn);
        st64(p64, e, pn);
        v[3 * r] += tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y +
                    V.shift[r] * (pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y);
      }
    }
  } else {
    using Lo = typename LoPtr<P>::T;
    const Lo* __restrict__ rh = reinterpret_cast<const Lo*>(P == PBF16 ? S.rh : S.r);
    const float4* __restrict__ r32 = reinterpret_cast<const float4*>(S.r);
    float4* __restrict__ t32 = reinterpret_cast<float4*>(S.t);
    float4* __restrict__ p32 = reinterpret_cast<float4*>(S.p);
    uint2* __restrict__ thb = reinterpret_cast<uint2*>(S.th);
    const M32* __restrict__ H = S.H32;
    const float* __restrict__ diag = S.diag32;
    // FP32 sums over the thread's sites (at most 32 terms); FP64 from the warp sum on
    float vf[R];
#pragma unroll
    for (int r = 0; r < R; r++) vf[r] = 0.f;
#pragma unroll 1
    for (int si = 0; si < spt; si++) {
      const int i = i0 + si * T;
      if (i >= Ns) break;
      const int jj[3] = {__ldg(V.nbr + i), __ldg(V.nbr + Ns + i), __ldg(V.nbr + 2 * Ns + i)};
      const M32 m[3] = {H[i], H[Ns + i], H[2 * Ns + i]};
      const float dg = __ldg(diag + i);
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (r >= nr || !act[r]) continue;
        const int e = i * R + r;
        const Sp32 self = ld32(r32, e);
        Sp32 o{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
#pragma unroll
        for (int k3 = 0; k3 < 3; k3++) {
          const Sp32 bk = LoField<P>::ld(rh, jj[k3] * R + r);
          o.s0 = cfmaf(make_float2(m[k3].r0.x, m[k3].r0.y), bk.s0, o.s0);
          o.s0 = cfmaf(make_float2(m[k3].r0.z, m[k3].r0.w), bk.s1, o.s0);
          o.s1 = cfmaf(make_float2(m[k3].r1.x, m[k3].r1.y), bk.s0, o.s1);
          o.s1 = cfmaf(make_float2(m[k3].r1.z, m[k3].r1.w), bk.s1, o.s1);
        }
        const Sp32 ti = ld32(t32, e), pi = ld32(p32, e);
        const float2 ar = make_float2(float(arx[r]), float(ary[r]));
        const float bt = float(beta[r]);
        Sp32 tn, pn;
        tn.s0 = cfmaf(ar, o.s0, make_float2(bt * ti.s0.x, bt * ti.s0.y));
        tn.s1 = cfmaf(ar, o.s1, make_float2(bt * ti.s1.x, bt * ti.s1.y));
        pn.s0 = cfmaf(ar, self.s0, make_float2(bt * pi.s0.x, bt * pi.s0.y));
        pn.s1 = cfmaf(ar, self.s1, make_float2(bt * pi.s1.x, bt * pi.s1.y));
        st32(t32, e, tn);
        if constexpr (P == PBF16) stbf(thb, e, tn);
        st32(p32, e, pn);
        const float tt = tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y;
        const float pp = pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y;
        vf[r] += tt + float(V.shift[r]) * pp;
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) v[3 * r] += double(vf[r]);
  }
}

// B: q = D^dag t;  r -= alpha (q + shift p);  x += alpha p;  v = |r|^2
template <int P, int R, int T>
__device__ __forceinline__ void tile_B(const BatchSys& S, int i0, int spt, const int* __restrict__ act,
                                       const double* __restrict__ alpha, S64* __restrict__ xa, double* v) {
  constexpr bool mixed = (P != P64);
  const TileView<R> V(S);
  const int Ns = V.Ns, nr = V.nr;
  if constexpr (!mixed) {
    S64* __restrict__ r64 = reinterpret_cast<S64*>(S.r);
    const S64* __restrict__ p64 = reinterpret_cast<const S64*>(S.p);
    const S64* __restrict__ t64w = reinterpret_cast<const S64*>(S.t);
    const M64* __restrict__ Hd = S.Hd;
    const double* __restrict__ diag = S.diag;
#pragma unroll 1
    for (int si = 0; si < spt; si++) {
      const int i = i0 + si * T;
      if (i >= Ns) break;
      const int jj[3] = {__ldg(V.nbr + i), __ldg(V.nbr + Ns + i), __ldg(V.nbr + 2 * Ns + i)};
      const M64 m[3] = {Hd[i], Hd[Ns + i], Hd[2 * Ns + i]};
      const double dg = __ldg(diag + i);
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (r >= nr || !act[r]) continue;
        const int e = i * R + r;
        const Sp64 self = ld64(t64w, e);
        Sp64 q{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
        for (int k3 = 0; k3 < 3; k3++) {
          const Sp64 bk = ld64(t64w, jj[k3] * R + r);
          q.s0 = cfma(m[k3].h00, bk.s0, q.s0);
          q.s0 = cfma(m[k3].h01, bk.s1, q.s0);
          q.s1 = cfma(m[k3].h10, bk.s0, q.s1);
          q.s1 = cfma(m[k3].h11, bk.s1, q.s1);
        }
        const Sp64 pi = ld64(p64, e), ri = ld64(r64, e), xi = ld64(xa, e);
        const double al = alpha[r], s = V.shift[r];
        Sp64 rn, xn;
        rn.s0 = csub(ri.s0, cscale(al, cadd(q.s0, cscale(s, pi.s0))));
        rn.s1 = csub(ri.s1, cscale(al, cadd(q.s1, cscale(s, pi.s1))));
        xn.s0 = cadd(xi.s0, cscale(al, pi.s0));
        xn.s1 = cadd(xi.s1, cscale(al, pi.s1));
        st64(r64, e, rn);
        st64(xa, e, xn);
        v[3 * r] += rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y;
      }
    }
  } else {
    using Lo = typename LoPtr<P>::T;
    const Lo* __restrict__ th = reinterpret_cast<const Lo*>(P == PBF16 ? S.th : S.t);
    const float4* __restrict__ t32 = reinterpret_cast<const float4*>(S.t);
    float4* __restrict__ r32 = reinterpret_cast<float4*>(S.r);
    const float4* __restrict__ p32 = reinterpret_cast<const float4*>(S.p);
    float4* __restrict__ xlo = reinterpret_cast<float4*>(S.xlo);
    uint2* __restrict__ rhb = reinterpret_cast<uint2*>(S.rh);
    const M32* __restrict__ Hd = S.Hd32;
    const float* __restrict__ diag = S.diag32;
    float vf[R];
#pragma unroll
    for (int r = 0; r < R; r++) vf[r] = 0.f;
#pragma unroll 1
    for (int si = 0; si < spt; si++) {
      const int i = i0 + si * T;
      if (i >= Ns) break;
      const int jj[3] = {__ldg(V.nbr + i), __ldg(V.nbr + Ns + i), __ldg(V.nbr + 2 * Ns + i)};
      const M32 m[3] = {Hd[i], Hd[Ns + i], Hd[2 * Ns + i]};
      const float dg = __ldg(diag + i);
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (r >= nr || !act[r]) continue;
        const int e = i * R + r;
        const Sp32 self = ld32(t32, e);
        Sp32 q{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
#pragma unroll
        for (int k3 = 0; k3 < 3; k3++) {
          const Sp32 bk = LoField<P>::ld(th, jj[k3] * R + r);
          q.s0 = cfmaf(make_float2(m[k3].r0.x, m[k3].r0.y), bk.s0, q.s0);
          q.s0 = cfmaf(make_float2(m[k3].r0.z, m[k3].r0.w), bk.s1, q.s0);
          q.s1 = cfmaf(make_float2(m[k3].r1.x, m[k3].r1.y), bk.s0, q.s1);
          q.s1 = cfmaf(make_float2(m[k3].r1.z, m[k3].r1.w), bk.s1, q.s1);
        }
        const Sp32 pi = ld32(p32, e), ri = ld32(r32, e), xi = ld32(xlo, e);
        const float al = float(alpha[r]), sf = float(V.shift[r]);
        Sp32 rn, xn;
        rn.s0 = make_float2(ri.s0.x - al * (q.s0.x + sf * pi.s0.x), ri.s0.y - al * (q.s0.y + sf * pi.s0.y));
        rn.s1 = make_float2(ri.s1.x - al * (q.s1.x + sf * pi.s1.x), ri.s1.y - al * (q.s1.y + sf * pi.s1.y));
        xn.s0 = make_float2(xi.s0.x + al * pi.s0.x, xi.s0.y + al * pi.s0.y);
        xn.s1 = make_float2(xi.s1.x + al * pi.s1.x, xi.s1.y + al * pi.s1.y);
        st32(r32, e, rn);
        if constexpr (P == PBF16) stbf(rhb, e, rn);
        st32(xlo, e, xn);
        vf[r] += rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y;
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) v[3 * r] += double(vf[r]);
  }
}

// INIT: |b|^2, x = 0, r = b, p = t = 0 (and the low-precision copies)
template <int P, int R, int T>
__device__ __forceinline__ void tile_init(const BatchSys& S, int i0, int spt, S64* xa, double* v) {
  constexpr bool mixed = (P != P64);
  const int Ns = S.Ns, nr = S.nrhs;
#pragma unroll 1
  for (int si = 0; si < spt; si++) {
    const int i = i0 + si * T;
    if (i >= Ns) break;
#pragma unroll 1
    for (int r = 0; r < nr; r++) {
      const int e = i * R + r;
      const Sp64 bi = ld64(S.b, e);
      v[3 * r] += bi.s0.x * bi.s0.x + bi.s0.y * bi.s0.y + bi.s1.x * bi.s1.x + bi.s1.y * bi.s1.y;
      const Sp64 z{make_double2(0, 0), make_double2(0, 0)};
      st64(xa, e, z);
      if constexpr (!mixed) {
        st64(reinterpret_cast<S64*>(S.r), e, bi);
        st64(reinterpret_cast<S64*>(S.p), e, z);
        st64(reinterpret_cast<S64*>(S.t), e, z);
      } else {
        const Sp32 bl{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
        const Sp32 zl{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        st32(reinterpret_cast<float4*>(S.r), e, bl);
        st32(reinterpret_cast<float4*>(S.t), e, zl);
        if constexpr (P == PBF16) {
          stbf(reinterpret_cast<uint2*>(S.rh), e, bl);
          stbf(reinterpret_cast<uint2*>(S.th), e, zl);
        }
        st32(reinterpret_cast<float4*>(S.p), e, zl);
        st32(reinterpret_cast<float4*>(S.xlo), e, zl);
      }
    }
  }
}

// R1: t64 = D (x_hi + x_lo);  x_hi2 = x_hi + x_lo
template <int P, int R, int T>
__device__ __forceinline__ void tile_R1(const BatchSys& S, int i0, int spt, const int* act, const S64* xa, S64* xb) {
  constexpr bool mixed = (P != P64);
  const int Ns = S.Ns, nr = S.nrhs;
  const float4* xlo = reinterpret_cast<const float4*>(S.xlo);
  auto xs = [&](int e) {
    const Sp64 h = ld64(xa, e);
    if constexpr (!mixed) {
      return h;
    } else {
      const Sp32 l = ld32(xlo, e);
      return Sp64{make_double2(h.s0.x + l.s0.x, h.s0.y + l.s0.y), make_double2(h.s1.x + l.s1.x, h.s1.y + l.s1.y)};
    }
  };
#pragma unroll 1
  for (int si = 0; si < spt; si++) {
    const int i = i0 + si * T;
    if (i >= Ns) break;
    const double dg = __ldg(S.diag + i);
#pragma unroll 1
    for (int r = 0; r < nr; r++) {
      const int e = i * R + r;
      if (!act[r]) {
        // a finished right-hand side keeps its solution across the buffer swap
        // that follows this phase
        if constexpr (mixed) st64(xb, e, ld64(xa, e));
        continue;
      }
      const Sp64 self = xs(e);
      st64(xb, e, self);
      Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll 1
      for (int k3 = 0; k3 < 3; k3++) {
        const M64 mk = S.H[k3 * Ns + i];
        const Sp64 bj = xs(__ldg(S.nbr + k3 * Ns + i) * R + r);
        o.s0 = cfma(mk.h00, bj.s0, o.s0);
        o.s0 = cfma(mk.h01, bj.s1, o.s0);
        o.s1 = cfma(mk.h10, bj.s0, o.s1);
        o.s1 = cfma(mk.h11, bj.s1, o.s1);
      }
      st64(S.t64, e, o);
    }
  }
}

// R2: r = b - D^dag t64 - shift x (FP64 true residual), its norm and <r, p>
template <int P, int R, int T>
__device__ __forceinline__ void tile_R2(const BatchSys& S, int i0, int spt, const int* act, const S64* xa, double* v) {
  constexpr bool mixed = (P != P64);
  const int Ns = S.Ns, nr = S.nrhs;
#pragma unroll 1
  for (int si = 0; si < spt; si++) {
    const int i = i0 + si * T;
    if (i >= Ns) break;
    const double dg = __ldg(S.diag + i);
#pragma unroll 1
    for (int r = 0; r < nr; r++) {
      if (!act[r]) continue;
      const int e = i * R + r;
      const Sp64 self = ld64(S.t64, e);
      Sp64 q{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll 1
      for (int k3 = 0; k3 < 3; k3++) {
        const M64 mk = S.Hd[k3 * Ns + i];
        const Sp64 bj = ld64(S.t64, __ldg(S.nbr + k3 * Ns + i) * R + r);
        q.s0 = cfma(mk.h00, bj.s0, q.s0);
        q.s0 = cfma(mk.h01, bj.s1, q.s0);
        q.s1 = cfma(mk.h10, bj.s0, q.s1);
        q.s1 = cfma(mk.h11, bj.s1, q.s1);
      }
      const Sp64 bi = ld64(S.b, e), xi = ld64(xa, e);
      const double s = S.shift[r];
      Sp64 rt;
      rt.s0 = csub(bi.s0, cadd(q.s0, cscale(s, xi.s0)));
      rt.s1 = csub(bi.s1, cadd(q.s1, cscale(s, xi.s1)));
      double2 pv0, pv1;
      if constexpr (!mixed) {
        const Sp64 pi = ld64(reinterpret_cast<const S64*>(S.p), e);
        pv0 = pi.s0;
        pv1 = pi.s1;
        st64(reinterpret_cast<S64*>(S.r), e, rt);
      } else {
        const Sp32 pi = ld32(reinterpret_cast<const float4*>(S.p), e);
        pv0 = make_double2(pi.s0.x, pi.s0.y);
        pv1 = make_double2(pi.s1.x, pi.s1.y);
        const Sp32 rl{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
        st32(reinterpret_cast<float4*>(S.r), e, rl);
        if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(S.rh), e, rl);
        st32(reinterpret_cast<float4*>(S.xlo), e, Sp32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)});
      }
      v[3 * r] += rt.s0.x * rt.s0.x + rt.s0.y * rt.s0.y + rt.s1.x * rt.s1.x + rt.s1.y * rt.s1.y;
      v[3 * r + 1] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
      v[3 * r + 2] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
    }
  }
}

// Register budgets: one right-hand side per system runs at 64 registers (1024
// threads per SM, a few bytes spilled); tiles of 2 and 4 take 128 (measured
// faster than 64 with their spills on the 256-right-hand-side batch); 8 up to 255.
template <int P, int R, int T>
__global__ void __launch_bounds__(T, (R == 1 ? 1024 / T : R <= 4 ? 512 / T : 256 / T)) k_batched_dyn(DynArgs a) {
  constexpr int NQ = 3 * R;
  constexpr int NW = T / 32;
  constexpr bool mixed = (P != P64);
  static_assert(NQ <= 32, "one warp finishes a system");
  // per-warp coefficients of the tile's system and the finisher's scratch
  __shared__ double s_beta[NW][R], s_arx[NW][R], s_ary[NW][R], s_alpha[NW][R];
  __shared__ int s_act[NW][R];
  __shared__ double s_red[NW][32];
  __shared__ double s_tot[NW][NQ];

  DynState<R>* ds = reinterpret_cast<DynState<R>*>(a.state);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  const unsigned long long NT = (unsigned long long)a.ntiles;
  bool aborted = false;

  // work item = step * ntiles + tile, taken in increasing order; the next one
  // is fetched while the current one is worked on
  unsigned long long next = 0;
  if (lane == 0) next = atomicAdd(a.work, 1ull);
  while (true) {
    const unsigned long long item = __shfl_sync(full, next, 0);
    const int step = int(item / NT);
    const int g = int(item - (unsigned long long)step * NT);
    const int sidx = __ldg(a.sys_of_tile + g);
    const BatchSys& S = a.sys[sidx];
    volatile DynState<R>* d = ds + sidx;
    int st = D_DONE, xsel = 0, quit = 0;
    if (lane == 0) {
      next = atomicAdd(a.work, 1ull);
      // wait until this system has finished step - 1: then its state is the
      // one of this step (a finished system's tiles are skipped)
      const int wr = wait_step(a.epoch + sidx, step, &d->state, D_DONE, &a.bar->abort, a.spin_limit);
      if (wr == 0) st = d->state;
      if (wr == 2) quit = 2;
      if (!quit) {
        if (st == D_DONE) {
          atomicMax(a.work, (unsigned long long)step * NT + (unsigned long long)S.ch1);  // skip its other tiles
          if (ld_volatile_int(a.ndone) >= a.nsys) quit = 1;  // every system finished: leave
        } else {
          xsel = d->xsel;
        }
      }
    }
    quit = __shfl_sync(full, quit, 0);
    if (quit) {
      aborted = quit == 2;
      break;
    }
    st = __shfl_sync(full, st, 0);
    xsel = __shfl_sync(full, xsel, 0);
    __syncwarp();  // orders lane 0's acquire before the other lanes' loads
    if (st == D_DONE) continue;
    if (lane < R) {
      s_act[w][lane] = d->active[lane];
      s_beta[w][lane] = d->beta[lane];
      s_arx[w][lane] = d->a_r[lane].x;
      s_ary[w][lane] = d->a_r[lane].y;
      s_alpha[w][lane] = d->alpha[lane];
    }
    __syncwarp();

    S64* xa = xsel ? S.xhi2 : S.xhi;
    double v[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) v[q] = 0.0;
    const int i0 = (g - S.ch0) * 32 * a.spt + lane;
    if (st == D_A) {
      tile_A<P, R, 32>(S, i0, a.spt, s_act[w], s_beta[w], s_arx[w], s_ary[w], v);
    } else if (st == D_B) {
      tile_B<P, R, 32>(S, i0, a.spt, s_act[w], s_alpha[w], xa, v);
    } else if (st == D_INIT) {
      tile_init<P, R, 32>(S, i0, a.spt, xa, v);
    } else if (st == D_R1) {
      tile_R1<P, R, 32>(S, i0, a.spt, s_act[w], xa, xsel ? S.xhi : S.xhi2);
    } else if (st == D_R2) {
      tile_R2<P, R, 32>(S, i0, a.spt, s_act[w], xa, v);
    }
    // ---- the tile's partial sums into its slot; the last tile of the system finishes the step
    if (st == D_R2) {
#pragma unroll
      for (int q = 0; q < NQ; q++) v[q] = warp_sum(v[q]);
    } else {  // the other phases sum one norm per right-hand side
#pragma unroll
      for (int r = 0; r < R; r++) v[3 * r] = warp_sum(v[3 * r]);
    }
    int fin = 0;
    if (lane == 0) {
      double* pp = a.part + size_t(g) * NQ;
#pragma unroll
      for (int q = 0; q < NQ; q++) __stcg(pp + q, v[q]);
      __threadfence();
      const int prev = atomicAdd(a.sys_cnt + sidx, 1);
      fin = (prev == S.ch1 - S.ch0 - 1);
    }
    fin = __shfl_sync(full, fin, 0);
    if (fin) {
      __threadfence();
      // the system's totals from its tile slots, in a fixed order: lane l sums
      // value l % nq of tiles l / nq, l / nq + 32 / nq, ... (four loads in
      // flight), then lane q adds the lanes of value q in lane order.  Only
      // the R2 step has three values per right-hand side; the others one.
      const int nt = S.ch1 - S.ch0;
      const int nq = st == D_R2 ? NQ : R, stride = st == D_R2 ? 1 : 3;
      const int tl = 32 / nq, used = tl * nq;
      double acc = 0.0;
      if (lane < used) {
        const double* base = a.part + size_t(S.ch0) * NQ + (lane % nq) * stride;
        int t = lane / nq;
        for (; t + 3 * tl < nt; t += 4 * tl) {
          const double x0 = __ldcg(base + size_t(t) * NQ), x1 = __ldcg(base + size_t(t + tl) * NQ),
                       x2 = __ldcg(base + size_t(t + 2 * tl) * NQ), x3 = __ldcg(base + size_t(t + 3 * tl) * NQ);
          acc += x0;
          acc += x1;
          acc += x2;
          acc += x3;
        }
        for (; t < nt; t += tl) acc += __ldcg(base + size_t(t) * NQ);
      }
      s_red[w][lane] = acc;
      __syncwarp();
      if (lane < NQ) s_tot[w][lane] = 0.0;
      __syncwarp();
      if (lane < nq) {
        double t = 0.0;
        for (int j = lane; j < used; j += nq) t += s_red[w][j];
        s_tot[w][lane * stride] = t;
      }
      __syncwarp();
      if (lane == 0) {
        a.sys_cnt[sidx] = 0;
        dyn_transition<R>(a, S, sidx, d, s_tot[w], mixed, a.ndone);
        __threadfence();
        st_release_s32(a.epoch + sidx, step + 1);  // the system's next step may start
      }
      __syncwarp();
    }
  }
  if (aborted && lane == 0) {
    const int gw = blockIdx.x * NW + w, nw = gridDim.x * NW;
    for (int s2 = gw; s2 < a.nsys; s2 += nw) atomicCAS(a.status + s2, -1, QED3_ERR_TIMEOUT);
  }
}

template <int P, int R>
const void* dyn_kernel(int threads) {
  return threads == 128 ? (const void*)k_batched_dyn<P, R, 128> : (const void*)k_batched_dyn<P, R, 256>;
}

template <int P, int R>
int dyn_launch(DynArgs& args, int grid, int threads, cudaStream_t st) {
  void* kargs[] = {&args};
  QED3_CUDA_TRY(cudaLaunchCooperativeKernel(dyn_kernel<P, R>(threads), dim3(grid), dim3(threads), kargs, 0, st));
  return QED3_OK;
}

template <int P, int R>
int dyn_occupancy(int threads, int* per_sm) {
  QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, dyn_kernel<P, R>(threads), threads, 0));
  return QED3_OK;
}

#define QED3_DYN_DISPATCH(P, R, fn, ...) \
  (R == 1 ? fn<P, 1>(__VA_ARGS__) : R == 2 ? fn<P, 2>(__VA_ARGS__) : R == 4 ? fn<P, 4>(__VA_ARGS__) : fn<P, 8>(__VA_ARGS__))

}  // namespace

int batch_dyn_occupancy(int prec, int R, int threads, int* per_sm) {
  if (prec == QED3_PREC_F64) return QED3_DYN_DISPATCH(P64, R, dyn_occupancy, threads, per_sm);
  if (prec == QED3_PREC_F32) return QED3_DYN_DISPATCH(P32, R, dyn_occupancy, threads, per_sm);
  return QED3_DYN_DISPATCH(PBF16, R, dyn_occupancy, threads, per_sm);
}

int batch_dyn_launch(int prec, int R, DynArgs& args, int grid, int threads, cudaStream_t st) {
  if (prec == QED3_PREC_F64) return QED3_DYN_DISPATCH(P64, R, dyn_launch, args, grid, threads, st);
  if (prec == QED3_PREC_F32) return QED3_DYN_DISPATCH(P32, R, dyn_launch, args, grid, threads, st);
  return QED3_DYN_DISPATCH(PBF16, R, dyn_launch, args, grid, threads, st);
}

}  // namespace qed3
