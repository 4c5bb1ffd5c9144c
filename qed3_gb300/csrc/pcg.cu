// Preconditioned persistent CG with the learned block-local preconditioner.
//
// No counterpart in the reference (its solvers are unpreconditioned CG,
// src/both_3d/sparse_matrix.h / cg_cuda.h).  Same skeleton as the
// register-resident solver (solver_v2.cu): one block per SM, thread t of block
// b owns sites b*per + k*T + t, two grid barriers per iteration, FP64
// reductions riding on them, fp32 state with fp32/bf16 halo copies, FP64
// reliable updates and an FP64 true-residual certificate.  What changes:
//
//   z = N r is applied right after r is updated, inside phase B, entirely in
//   shared memory: N = a^2 I + sum_{w,w'} O_w^dag M_{ww'} O_w' with words
//   O_w over {Hd, Ho} (the spin-diagonal / off-diagonal parts of the Dirac hop
//   restricted to the block) -- it never leaves the SM, so the iteration
//   keeps its two grid barriers.  N is hermitian positive definite, so the
//   short PCG recurrence holds:
//     t = D p = a_z D z + beta t,  p = a_z z + beta p   (phase A, gathers z)
//     q = D^dag t + s p, x += alpha p, r -= alpha q, z = N r   (phase B, gathers t)
//   with alpha = <r,z> / (|t|^2 + s|p|^2), beta = <r,z>_new / <r,z>_old.
//   After a reliable update (r = b - A x in FP64) the direction is
//   re-conjugated to the new residual: a_z = 1 - beta <r,p> / <r,z>.

#include <cmath>
#include <string>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"
#include "lpc_impl.h"
#include "pcg_impl.h"
#include "v2_common.cuh"

namespace qed3 {

struct PcgArgs {
  int Ns, per;
  const int* nbr;
  const M64* H;
  const M64* Hd;
  const double* diag;
  const M32* H32;
  const M32* Hd32;
  const float* diag32;
  const S64* b;
  S64* x;
  S64* t64;
  void* halo_z;
  void* halo_t;
  double* partials;
  GridBar2* bar;
  double* scal;
  double tol2, delta2, shift;
  int maxiter;
  int flexible;  // Polak-Ribiere beta
  long long spin_limit;
  LpcWordCoef pc;
  // pipelined kernel: gathered copies of u, p, q at residual replacements
  void* halo_u;
  void* halo_p;
  void* halo_q;
};

__device__ __forceinline__ float4 sp2f4(const Sp32& v) { return make_float4(v.s0.x, v.s0.y, v.s1.x, v.s1.y); }
__device__ __forceinline__ Sp32 f42sp(const float4& v) { return {make_float2(v.x, v.y), make_float2(v.z, v.w)}; }

// Hop blocks of the owned sites: from shared memory (HS, staged once per
// solve, SoA Hs[(2k + row) * per + loc]) or through the read-only path.
template <bool HS>
__device__ __forceinline__ void ldH(const M32* __restrict__ Hg, const float4* Hs, int per, int Ns, int k, int i,
                                    int loc, float4& r0, float4& r1) {
  if constexpr (HS) {
    r0 = Hs[(2 * k) * per + loc];
    r1 = Hs[(2 * k + 1) * per + loc];
  } else {
    const float4* m = reinterpret_cast<const float4*>(Hg + size_t(k) * Ns + i);
    r0 = __ldg(m);
    r1 = __ldg(m + 1);
  }
}

__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }
// Hd y = (h00 y0, h11 y1), Ho y = (h01 y1, h10 y0) accumulated into d / o
__device__ __forceinline__ void acc_d(Sp32& d, const float4& r0, const float4& r1, const float4& y) {
  d.s0 = cfmaf(lo2(r0), lo2(y), d.s0);
  d.s1 = cfmaf(hi2(r1), hi2(y), d.s1);
}
__device__ __forceinline__ void acc_o(Sp32& o, const float4& r0, const float4& r1, const float4& y) {
  o.s0 = cfmaf(hi2(r0), hi2(y), o.s0);
  o.s1 = cfmaf(lo2(r1), lo2(y), o.s1);
}

// One pass over the in-block neighbours of owned site i (block-local index
// loc): reads every hop block once and applies it to NF shared-memory fields;
// MODE[f] = 1: Hd F_f -> out[f], 2: Ho F_f -> out[f], 3: both -> out[f], out[f + NF].
template <bool HS, int NF>
__device__ __forceinline__ void hop_pass(const float4* const (&F)[NF], const int (&mode)[NF], const int (&jj)[3],
                                         int blk0, int per, int i, int loc, int Ns, const M32* __restrict__ Hg,
                                         const float4* Hs, Sp32 (&out)[2 * NF]) {
#pragma unroll
  for (int f = 0; f < 2 * NF; f++) out[f] = Sp32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int l = jj[k] - blk0;
    if (unsigned(l) >= unsigned(per)) continue;
    float4 r0, r1;
    ldH<HS>(Hg, Hs, per, Ns, k, i, loc, r0, r1);
#pragma unroll
    for (int f = 0; f < NF; f++) {
      const float4 y = F[f][l];
      if (mode[f] == 1) acc_d(out[f], r0, r1, y);
      else if (mode[f] == 2) acc_o(out[f], r0, r1, y);
      else {
        acc_d(out[f], r0, r1, y);
        acc_o(out[f + NF], r0, r1, y);
      }
    }
  }
}

__device__ __forceinline__ void acc_c(Sp32& acc, float2 c, const Sp32& f) {
  acc.s0 = cfmaf(c, f.s0, acc.s0);
  acc.s1 = cfmaf(c, f.s1, acc.s1);
}
__device__ __forceinline__ Sp32 sp_add(const Sp32& a, const Sp32& b, float sb) {
  return {make_float2(a.s0.x + sb * b.s0.x, a.s0.y + sb * b.s0.y), make_float2(a.s1.x + sb * b.s1.x, a.s1.y + sb * b.s1.y)};
}

// z = N r for the block's sites; every thread of the block calls it (sites
// past Ns carry zeros).  S: NW fields of `per` float4 in shared memory.
//   f = (r, Hd r, Ho r, Hd Hd r, Hd Ho r, Ho Hd r, Ho Ho r),  g = M f,
//   z = a^2 r + g0 + Hd u + Ho v,  u = g1 + Hd g3 - Ho g5,  v = -g2 - Hd g4 + Ho g6
// (the adjoint words, using Hd^dag = Hd and Ho^dag = -Ho): four neighbour passes.
template <int NW, int SPT, bool HS>
__device__ __forceinline__ void pc_apply(const PcgArgs& a, float4* S, const float4* Hs, int blk0,
                                         const int (&own)[SPT], const int (&loc)[SPT], const bool (&val)[SPT],
                                         const int (&jj)[SPT][3], const Sp32 (&r)[SPT], Sp32 (&z)[SPT]) {
  const int per = a.per, Ns = a.Ns;
  const Sp32 zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  float4* S0 = S;
  float4* S1 = S + per;
  float4* S2 = S + 2 * per;
#pragma unroll
  for (int k = 0; k < SPT; k++) S0[loc[k]] = sp2f4(val[k] ? r[k] : zero);
  __syncthreads();
  Sp32 g0[SPT], g1[SPT], g2[SPT];
  if constexpr (NW == 7) {
    float4* S3 = S + 3 * per;
    float4* S4 = S + 4 * per;
    float4* S5 = S + 5 * per;
    float4* S6 = S + 6 * per;
#pragma unroll
    for (int k = 0; k < SPT; k++) {
      Sp32 o[2];
      o[0] = o[1] = zero;
      if (val[k]) {
        const float4* const F[1] = {S0};
        const int md[1] = {3};
        hop_pass<HS, 1>(F, md, jj[k], blk0, per, own[k], loc[k], Ns, a.H32, Hs, o);
      }
      S1[loc[k]] = sp2f4(o[0]);  // Hd r
      S2[loc[k]] = sp2f4(o[1]);  // Ho r
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SPT; k++) {
      Sp32 o[4];
      o[0] = o[1] = o[2] = o[3] = zero;
      if (val[k]) {
        const float4* const F[2] = {S1, S2};
        const int md[2] = {3, 3};
        hop_pass<HS, 2>(F, md, jj[k], blk0, per, own[k], loc[k], Ns, a.H32, Hs, o);
      }
      // park the length-2 words in this site's own slots (f3 = Hd Hd r, f4 = Hd Ho r,
      // f5 = Ho Hd r, f6 = Ho Ho r), then stream the seven words through the 7 x 7
      // product one at a time; g3..g6 replace them in the same own slots
      S3[loc[k]] = sp2f4(o[0]);
      S4[loc[k]] = sp2f4(o[1]);
      S5[loc[k]] = sp2f4(o[2]);
      S6[loc[k]] = sp2f4(o[3]);
      Sp32 g[7];
#pragma unroll
      for (int w = 0; w < 7; w++) g[w] = zero;
#pragma unroll
      for (int qw = 0; qw < 7; qw++) {
        const Sp32 f = qw == 0 ? r[k] : f42sp((S + qw * per)[loc[k]]);
#pragma unroll
        for (int w = 0; w < 7; w++) acc_c(g[w], a.pc.M[w][qw], f);
      }
      g0[k] = g[0];
      g1[k] = g[1];
      g2[k] = g[2];
      S3[loc[k]] = sp2f4(g[3]);
      S4[loc[k]] = sp2f4(g[4]);
      S5[loc[k]] = sp2f4(g[5]);
      S6[loc[k]] = sp2f4(g[6]);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SPT; k++) {
      Sp32 u = zero, v = zero;
      if (val[k]) {
        Sp32 o[8];
        const float4* const F[4] = {S3, S4, S5, S6};
        const int md[4] = {1, 1, 2, 2};
        hop_pass<HS, 4>(F, md, jj[k], blk0, per, own[k], loc[k], Ns, a.H32, Hs, o);
        // o[0] = Hd g3, o[1] = Hd g4, o[2] = Ho g5, o[3] = Ho g6
        u = sp_add(sp_add(g1[k], o[0], 1.f), o[2], -1.f);
        v = sp_add(sp_add(sp_add(zero, g2[k], -1.f), o[1], -1.f), o[3], 1.f);
      }
      S1[loc[k]] = sp2f4(u);
      S2[loc[k]] = sp2f4(v);
    }
  } else {
#pragma unroll
    for (int k = 0; k < SPT; k++) {
      Sp32 f[3];
      f[0] = r[k];
      Sp32 o[2];
      o[0] = o[1] = zero;
      if (val[k]) {
        const float4* const F[1] = {S0};
        const int md[1] = {3};
        hop_pass<HS, 1>(F, md, jj[k], blk0, per, own[k], loc[k], Ns, a.H32, Hs, o);
      }
      f[1] = o[0];
      f[2] = o[1];
#pragma unroll
      for (int w = 0; w < 3; w++) {
        Sp32 g = zero;
#pragma unroll
        for (int q = 0; q < 3; q++) acc_c(g, a.pc.M[w][q], f[q]);
        if (w == 0) g0[k] = g;
        if (w == 1) g1[k] = g;
        if (w == 2) g2[k] = g;
      }
      S1[loc[k]] = sp2f4(val[k] ? g1[k] : zero);
      S2[loc[k]] = sp2f4(val[k] ? sp_add(zero, g2[k], -1.f) : zero);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < SPT; k++) {
    if (!val[k]) {
      z[k] = zero;
      continue;
    }
    Sp32 o[4];
    const float4* const F[2] = {S1, S2};
    const int md[2] = {1, 2};
    hop_pass<HS, 2>(F, md, jj[k], blk0, per, own[k], loc[k], Ns, a.H32, Hs, o);
    Sp32 zz = sp_add(g0[k], r[k], a.pc.a2);
    zz = sp_add(sp_add(zz, o[0], 1.f), o[1], 1.f);
    z[k] = zz;
  }
}

// own-site stencil o = diag * self + sum_k H_k halo[nbr_k], hop blocks from
// shared memory (HS) or the read-only path
template <int P, bool HS>
__device__ __forceinline__ Sp32 stencil32h(int i, int loc, int per, int Ns, const int (&jj)[3],
                                           const M32* __restrict__ Hg, const float4* Hs, float dg, const Sp32& self,
                                           const void* halo) {
  Sp32 o{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
  const Sp32 b0 = hl32<P>(halo, jj[0]), b1 = hl32<P>(halo, jj[1]), b2 = hl32<P>(halo, jj[2]);
  const Sp32 bs[3] = {b0, b1, b2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float4 r0, r1;
    ldH<HS>(Hg, Hs, per, Ns, k, i, loc, r0, r1);
    o.s0 = cfmaf(lo2(r0), bs[k].s0, o.s0);
    o.s0 = cfmaf(hi2(r0), bs[k].s1, o.s0);
    o.s1 = cfmaf(lo2(r1), bs[k].s0, o.s1);
    o.s1 = cfmaf(hi2(r1), bs[k].s1, o.s1);
  }
  return o;
}

__device__ __forceinline__ float rdotf(const Sp32& a, const Sp32& b) {  // Re <a, b>
  return a.s0.x * b.s0.x + a.s0.y * b.s0.y + a.s1.x * b.s1.x + a.s1.y * b.s1.y;
}

// Dynamic shared memory: NW fields of `per` float4 for the preconditioner,
// one for q (flexible mode), then (HS) the owned sites' hop blocks of D and
// D^dag, 6 x per float4 each.
template <int P, int NW, int SPT>
__global__ void __launch_bounds__(576, 1) k_pcg(PcgArgs a) {
  constexpr bool HS = (SPT == 1);
  extern __shared__ float4 S[];
  __shared__ double sh[32 * 4 + 64 + 8];
  const int Ns = a.Ns;
  const int T = blockDim.x;
  const int blk0 = blockIdx.x * a.per;
  float4* Sq = S + NW * a.per;        // q of the owned sites (flexible mode)
  float4* HsD = Sq + a.per;           // hop blocks of D (own sites)
  float4* HsDd = HsD + 6 * a.per;     // hop blocks of D^dag
  float dg[SPT];

  int own[SPT], loc[SPT];
  bool val[SPT];
  int jj[SPT][3];
  Sp32 r[SPT], p[SPT], t[SPT], z[SPT];
  Sp64 xh[SPT];
  Sp32 xl[SPT];
  const Sp64 z64{make_double2(0, 0), make_double2(0, 0)};
  const Sp32 z32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};

  // ---- phase 0: ids, r = b, z = N r, p = t = x = 0 -------------------------------------
  double v2[2] = {0.0, 0.0};
#pragma unroll
  for (int k = 0; k < SPT; k++) {
    loc[k] = k * T + threadIdx.x;
    const int i = blk0 + loc[k];
    own[k] = i;
    val[k] = i < Ns;
    xh[k] = z64;
    xl[k] = z32;
    p[k] = z32;
    t[k] = z32;
    r[k] = z32;
#pragma unroll
    for (int q = 0; q < 3; q++) jj[k][q] = 0;
    dg[k] = 0.f;
    if constexpr (HS) {
#pragma unroll
      for (int q = 0; q < 6; q++) {
        const float4 zf = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4* mh = reinterpret_cast<const float4*>(a.H32 + size_t(q >> 1) * Ns + i) + (q & 1);
        const float4* md = reinterpret_cast<const float4*>(a.Hd32 + size_t(q >> 1) * Ns + i) + (q & 1);
        HsD[q * a.per + loc[k]] = val[k] ? __ldg(mh) : zf;
        HsDd[q * a.per + loc[k]] = val[k] ? __ldg(md) : zf;
      }
    }
    if (val[k]) {
      dg[k] = __ldg(a.diag32 + i);
#pragma unroll
      for (int q = 0; q < 3; q++) jj[k][q] = __ldg(a.nbr + q * Ns + i);
      const Sp64 bi = ld64(a.b, i);
      v2[0] += n2(bi);
      r[k] = Sp32{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
    }
  }
  pc_apply<NW, SPT, HS>(a, S, HsD, blk0, own, loc, val, jj, r, z);
#pragma unroll
  for (int k = 0; k < SPT; k++) {
    if (!val[k]) continue;
    hs32<P>(a.halo_z, own[k], z[k]);
    v2[1] += double(rdotf(r[k], z[k]));
  }
  unsigned int epoch = 0;
  int parity = 0;
  v2_publish<2>(v2, a.partials, parity, sh);
  if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
  {
    double tot[2];
    v2_total<2>(a.partials, parity, tot, sh);
    parity ^= 1;
    const double bnorm2 = tot[0];
    double rho = tot[1];
    double mu = bnorm2, mu_max = bnorm2, beta = 0.0, mu_true = bnorm2;
    double2 a_z = make_double2(1.0, 0.0);
    int iter = 0, nru = 0, status = QED3_ERR_NOCONV;
    const double s = a.shift;
    if (bnorm2 == 0.0) {
      status = QED3_OK;
      mu_true = 0.0;
      goto finish;
    }
    while (true) {
      // ---- phase A: t = a_z D z + beta t, p = a_z z + beta p ----------------------------
      {
        float v[1] = {0.f};
        const float2 az = make_float2(float(a_z.x), float(a_z.y));
        const float bt = float(beta);
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const int i = own[k];
          const Sp32 dz = stencil32h<P, HS>(i, loc[k], a.per, Ns, jj[k], a.H32, HsD, dg[k], z[k], a.halo_z);
          t[k].s0 = cfmaf(az, dz.s0, make_float2(bt * t[k].s0.x, bt * t[k].s0.y));
          t[k].s1 = cfmaf(az, dz.s1, make_float2(bt * t[k].s1.x, bt * t[k].s1.y));
          p[k].s0 = cfmaf(az, z[k].s0, make_float2(bt * p[k].s0.x, bt * p[k].s0.y));
          p[k].s1 = cfmaf(az, z[k].s1, make_float2(bt * p[k].s1.x, bt * p[k].s1.y));
          hs32<P>(a.halo_t, i, t[k]);
          v[0] += n2f(t[k]) + float(s) * n2f(p[k]);
        }
        v2_publish_f<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double gam[1];
      v2_total<1>(a.partials, parity, gam, sh);
      parity ^= 1;
      const double alpha = rho / gam[0];
      // ---- phase B: q = D^dag t + s p, x += alpha p, r -= alpha q, z = N r -------------
      {
        float v[3] = {0.f, 0.f, 0.f};
        const float al = float(alpha), sf = float(s);
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          const Sp32 q = stencil32h<P, HS>(own[k], loc[k], a.per, Ns, jj[k], a.Hd32, HsDd, dg[k], t[k], a.halo_t);
          const Sp32 qf = sp_add(q, p[k], sf);
          if (a.flexible) Sq[loc[k]] = sp2f4(qf);  // kept for <z', q> after the preconditioner
          r[k] = sp_add(r[k], qf, -al);
          xl[k] = sp_add(xl[k], p[k], al);
        }
        pc_apply<NW, SPT, HS>(a, S, HsD, blk0, own, loc, val, jj, r, z);
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          hs32<P>(a.halo_z, own[k], z[k]);
          v[0] += n2f(r[k]);
          v[1] += rdotf(r[k], z[k]);
          if (a.flexible) v[2] += rdotf(z[k], f42sp(Sq[loc[k]]));
        }
        if (a.flexible) v2_publish_f<3>(v, a.partials, parity, sh);
        else {
          float v2r[2] = {v[0], v[1]};
          v2_publish_f<2>(v2r, a.partials, parity, sh);
        }
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double mun[3] = {0.0, 0.0, 0.0};
      if (a.flexible) v2_total<3>(a.partials, parity, mun, sh);
      else {
        double m2[2];
        v2_total<2>(a.partials, parity, m2, sh);
        mun[0] = m2[0];
        mun[1] = m2[1];
      }
      parity ^= 1;
      iter++;
      const double mu_new = mun[0], rho_new = mun[1];
      mu_max = fmax(mu_max, mu_new);
      const bool want = !isfinite(mu_new) || !isfinite(alpha) || !(rho_new > 0.0) || mu_new < a.tol2 * bnorm2 ||
                        iter >= a.maxiter || mu_new < a.delta2 * mu_max;
      if (!want) {
        // flexible: <z', r' - r> = -alpha <z', q>
        beta = a.flexible ? -alpha * mun[2] / rho : rho_new / rho;
        a_z = make_double2(1.0, 0.0);
        rho = rho_new;
        mu = mu_new;
        continue;
      }
      // ---- R0: fold x, publish it ---------------------------------------------------------
#pragma unroll
      for (int k = 0; k < SPT; k++) {
        if (!val[k]) continue;
        xh[k].s0 = make_double2(xh[k].s0.x + xl[k].s0.x, xh[k].s0.y + xl[k].s0.y);
        xh[k].s1 = make_double2(xh[k].s1.x + xl[k].s1.x, xh[k].s1.y + xl[k].s1.y);
        xl[k] = z32;
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
      // ---- R2: r = b - D^dag t64 - s x, z = N r;  |r|^2, <r,z>, <r,p> --------------------
      {
        double v[4] = {0.0, 0.0, 0.0, 0.0};
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
          const double2 pv0 = make_double2(p[k].s0.x, p[k].s0.y), pv1 = make_double2(p[k].s1.x, p[k].s1.y);
          v[2] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
          v[3] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
          r[k] = Sp32{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
        }
        pc_apply<NW, SPT, HS>(a, S, HsD, blk0, own, loc, val, jj, r, z);
#pragma unroll
        for (int k = 0; k < SPT; k++) {
          if (!val[k]) continue;
          hs32<P>(a.halo_z, own[k], z[k]);
          v[1] += double(rdotf(r[k], z[k]));
        }
        v2_publish<4>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double tr[4];
      v2_total<4>(a.partials, parity, tr, sh);
      parity ^= 1;
      nru++;
      mu_true = tr[0];
      if (mu_true < a.tol2 * bnorm2) {
        status = QED3_OK;
        break;
      }
      if (iter >= a.maxiter || !isfinite(mu_true) || !(tr[1] > 0.0)) {
        status = QED3_ERR_NOCONV;
        break;
      }
      beta = tr[1] / rho;
      a_z = make_double2(1.0 - beta * tr[2] / tr[1], -beta * tr[3] / tr[1]);
      rho = tr[1];
      mu = mu_true;
      mu_max = mu_true;
    }
  finish:
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
    (void)mu;
    return;
  }
timeout:
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[4] = QED3_ERR_TIMEOUT;
    a.scal[5] = 0;
  }
}

// ---------------------------------------------------------------------------
// Streaming preconditioned CG for lattices that do not fit the registers
// ---------------------------------------------------------------------------
// Same recurrence, reliable updates and certificate as k_pcg, for lattices
// whose per-SM share exceeds what one block can hold in registers (about
// n >= 94): the preconditioner's blocks become tiles of `per` <= 512 sites,
// every block of a persistent one-block-per-SM grid walks its tiles inside
// each phase, and the solver state lives in global memory (read and written
// once per site and phase; the operator's hop blocks come through the
// read-only path).  z = N r is applied tile by tile in shared memory right
// after the tile's residual update, so an iteration keeps its two grid
// barriers; the tile's hop blocks are staged in shared memory for the four
// neighbour passes of N.  State arrays (internal order): r, p, t and z in
// FP32 (float4 per site), the gathered copies of z and t in the halo
// precision, x as an FP32 increment folded into FP64 at reliable updates.
struct PcgsState {
  float4* r;
  float4* p;
  float4* t;  // own FP32 copy of t (halo_t holds the gathered copy)
  float4* z;  // own FP32 copy of z
  float4* xl;
};

__device__ __forceinline__ Sp32 ldf4(const float4* f, int i) { return f42sp(__ldcg(f + i)); }
__device__ __forceinline__ void stf4(float4* f, int i, const Sp32& v) { __stcg(f + i, sp2f4(v)); }
// z and t: with FP32 halos the gathered copy is the FP32 value itself, so the
// own copy is not stored twice
template <int P>
__device__ __forceinline__ Sp32 own_ld(const float4* own, const void* halo, int i) {
  if constexpr (P == P32) return hl32<P>(halo, i);
  else return ldf4(own, i);
}
template <int P>
__device__ __forceinline__ void own_st(float4* own, void* halo, int i, const Sp32& v) {
  hs32<P>(halo, i, v);
  if constexpr (P != P32) stf4(own, i, v);
}

template <int P, int NW>
__global__ void __launch_bounds__(512, 1) k_pcgs(PcgArgs a, PcgsState st) {
  extern __shared__ float4 S[];
  __shared__ double sh[32 * 4 + 64 + 8];
  const int Ns = a.Ns, per = a.per;
  float4* Hs = S + NW * per;  // the tile's own hop blocks of D, read by the preconditioner's passes
  const int ntiles = (Ns + per - 1) / per;
  const Sp64 z64{make_double2(0, 0), make_double2(0, 0)};
  const Sp32 z32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  // per-tile site data of this thread
  auto site = [&](int tile, int (&own)[1], int (&loc)[1], bool (&val)[1], int (&jj)[1][3]) {
    loc[0] = threadIdx.x;
    own[0] = tile * per + threadIdx.x;
    val[0] = own[0] < Ns;
#pragma unroll
    for (int q = 0; q < 3; q++) jj[0][q] = val[0] ? __ldg(a.nbr + q * Ns + own[0]) : 0;
    // stage this site's hop blocks for the preconditioner (visible after its first __syncthreads)
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const float4* mh = reinterpret_cast<const float4*>(a.H32 + size_t(q >> 1) * Ns + own[0]) + (q & 1);
      Hs[q * per + loc[0]] = val[0] ? __ldg(mh) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  // ---- phase 0: r = b, z = N r, p = t = x = 0 ---------------------------------------------
  double v2[2] = {0.0, 0.0};
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int own[1], loc[1], jj[1][3];
    bool val[1];
    site(tile, own, loc, val, jj);
    Sp32 r[1] = {z32}, z[1];
    const int i = own[0];
    if (val[0]) {
      const Sp64 bi = ld64(a.b, i);
      v2[0] += n2(bi);
      r[0] = Sp32{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
    }
    pc_apply<NW, 1, true>(a, S, Hs, tile * per, own, loc, val, jj, r, z);
    if (val[0]) {
      stf4(st.r, i, r[0]);
      own_st<P>(st.z, a.halo_z, i, z[0]);
      stf4(st.p, i, z32);
      own_st<P>(st.t, a.halo_t, i, z32);
      stf4(st.xl, i, z32);
      hs64(a.x, i, z64);
      v2[1] += double(rdotf(r[0], z[0]));
    }
    __syncthreads();  // the tile's shared fields are reused by the next tile
  }
  unsigned int epoch = 0;
  int parity = 0;
  v2_publish<2>(v2, a.partials, parity, sh);
  if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
  {
    double tot[2];
    v2_total<2>(a.partials, parity, tot, sh);
    parity ^= 1;
    const double bnorm2 = tot[0];
    double rho = tot[1];
    double mu_max = bnorm2, beta = 0.0, mu_true = bnorm2;
    double2 a_z = make_double2(1.0, 0.0);
    int iter = 0, nru = 0, status = QED3_ERR_NOCONV;
    const double s = a.shift;
    if (bnorm2 == 0.0) {
      status = QED3_OK;
      mu_true = 0.0;
      goto finish;
    }
    while (true) {
      // ---- phase A: t = a_z D z + beta t, p = a_z z + beta p ----------------------------
      // two sites per thread in flight (this tile's and the next one's): all
      // their loads issue before the first dependent use
      {
        float v[1] = {0.f};
        const float2 az = make_float2(float(a_z.x), float(a_z.y));
        const float bt = float(beta);
        for (int tile = blockIdx.x; tile < ntiles; tile += 2 * gridDim.x) {
          int ii[2];
          bool ok[2];
          ii[0] = tile * per + threadIdx.x;
          ii[1] = (tile + gridDim.x) * per + threadIdx.x;
          ok[0] = ii[0] < Ns;
          ok[1] = tile + gridDim.x < ntiles && ii[1] < Ns;
          Sp32 dz[2], zi[2], ti[2], pi[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            if (!ok[u]) continue;
            const int i = ii[u];
            int jj[3];
#pragma unroll
            for (int q = 0; q < 3; q++) jj[q] = __ldg(a.nbr + q * Ns + i);
            zi[u] = own_ld<P>(st.z, a.halo_z, i);
            ti[u] = own_ld<P>(st.t, a.halo_t, i);
            pi[u] = ldf4(st.p, i);
            dz[u] = stencil32h<P, false>(i, 0, per, Ns, jj, a.H32, nullptr, __ldg(a.diag32 + i), zi[u], a.halo_z);
          }
#pragma unroll
          for (int u = 0; u < 2; u++) {
            if (!ok[u]) continue;
            const int i = ii[u];
            Sp32 t = ti[u], pp = pi[u];
            t.s0 = cfmaf(az, dz[u].s0, make_float2(bt * t.s0.x, bt * t.s0.y));
            t.s1 = cfmaf(az, dz[u].s1, make_float2(bt * t.s1.x, bt * t.s1.y));
            pp.s0 = cfmaf(az, zi[u].s0, make_float2(bt * pp.s0.x, bt * pp.s0.y));
            pp.s1 = cfmaf(az, zi[u].s1, make_float2(bt * pp.s1.x, bt * pp.s1.y));
            own_st<P>(st.t, a.halo_t, i, t);
            stf4(st.p, i, pp);
            v[0] += n2f(t) + float(s) * n2f(pp);
          }
        }
        v2_publish_f<1>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double gam[1];
      v2_total<1>(a.partials, parity, gam, sh);
      parity ^= 1;
      const double alpha = rho / gam[0];
      // ---- phase B1: q = D^dag t + s p, x += alpha p, r -= alpha q (two sites in flight) ------
      {
        const float al = float(alpha), sf = float(s);
        for (int tile = blockIdx.x; tile < ntiles; tile += 2 * gridDim.x) {
          int ii[2];
          bool ok[2];
          ii[0] = tile * per + threadIdx.x;
          ii[1] = (tile + gridDim.x) * per + threadIdx.x;
          ok[0] = ii[0] < Ns;
          ok[1] = tile + gridDim.x < ntiles && ii[1] < Ns;
          Sp32 q[2], pi[2], ri[2], xl[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            if (!ok[u]) continue;
            const int i = ii[u];
            int jj[3];
#pragma unroll
            for (int k = 0; k < 3; k++) jj[k] = __ldg(a.nbr + k * Ns + i);
            const Sp32 ti = own_ld<P>(st.t, a.halo_t, i);
            pi[u] = ldf4(st.p, i);
            ri[u] = ldf4(st.r, i);
            xl[u] = ldf4(st.xl, i);
            q[u] = stencil32h<P, false>(i, 0, per, Ns, jj, a.Hd32, nullptr, __ldg(a.diag32 + i), ti, a.halo_t);
          }
#pragma unroll
          for (int u = 0; u < 2; u++) {
            if (!ok[u]) continue;
            stf4(st.r, ii[u], sp_add(ri[u], sp_add(q[u], pi[u], sf), -al));
            stf4(st.xl, ii[u], sp_add(xl[u], pi[u], al));
          }
        }
      }
      // ---- phase B2: z = N r tile by tile (each thread reads back its own r) -------------
      {
        float v[2] = {0.f, 0.f};
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
          int own[1], loc[1], jj[1][3];
          bool val[1];
          site(tile, own, loc, val, jj);
          const int i = own[0];
          Sp32 r[1] = {z32}, z[1];
          if (val[0]) r[0] = ldf4(st.r, i);
          pc_apply<NW, 1, true>(a, S, Hs, tile * per, own, loc, val, jj, r, z);
          if (val[0]) {
            own_st<P>(st.z, a.halo_z, i, z[0]);
            v[0] += n2f(r[0]);
            v[1] += rdotf(r[0], z[0]);
          }
          __syncthreads();
        }
        v2_publish_f<2>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double mun[2];
      v2_total<2>(a.partials, parity, mun, sh);
      parity ^= 1;
      iter++;
      const double mu_new = mun[0], rho_new = mun[1];
      mu_max = fmax(mu_max, mu_new);
      const bool want = !isfinite(mu_new) || !isfinite(alpha) || !(rho_new > 0.0) || mu_new < a.tol2 * bnorm2 ||
                        iter >= a.maxiter || mu_new < a.delta2 * mu_max;
      if (!want) {
        beta = rho_new / rho;
        a_z = make_double2(1.0, 0.0);
        rho = rho_new;
        continue;
      }
      // ---- R0: fold x ---------------------------------------------------------------------
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * per + threadIdx.x;
        if (i >= Ns) continue;
        Sp64 xh = hl64(a.x, i);
        const Sp32 xl = ldf4(st.xl, i);
        xh.s0 = make_double2(xh.s0.x + xl.s0.x, xh.s0.y + xl.s0.y);
        xh.s1 = make_double2(xh.s1.x + xl.s1.x, xh.s1.y + xl.s1.y);
        hs64(a.x, i, xh);
        stf4(st.xl, i, z32);
      }
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R1: t64 = D x ------------------------------------------------------------------
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * per + threadIdx.x;
        if (i >= Ns) continue;
        int jj[3];
#pragma unroll
        for (int q = 0; q < 3; q++) jj[q] = __ldg(a.nbr + q * Ns + i);
        hs64(a.t64, i, stencil64(i, Ns, jj, a.H, a.diag, hl64(a.x, i), a.x));
      }
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R2: r = b - D^dag t64 - s x, z = N r;  |r|^2, <r,z>, <r,p> --------------------
      {
        double v[4] = {0.0, 0.0, 0.0, 0.0};
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
          int own[1], loc[1], jj[1][3];
          bool val[1];
          site(tile, own, loc, val, jj);
          const int i = own[0];
          Sp32 r[1] = {z32}, z[1];
          if (val[0]) {
            const Sp64 self = hl64(a.t64, i), xh = hl64(a.x, i);
            const Sp64 q = stencil64(i, Ns, jj[0], a.Hd, a.diag, self, a.t64);
            const Sp64 bi = ld64(a.b, i);
            Sp64 rt;
            rt.s0 = csub(bi.s0, cadd(q.s0, cscale(s, xh.s0)));
            rt.s1 = csub(bi.s1, cadd(q.s1, cscale(s, xh.s1)));
            v[0] += n2(rt);
            const Sp32 pf = ldf4(st.p, i);
            const double2 pv0 = make_double2(pf.s0.x, pf.s0.y), pv1 = make_double2(pf.s1.x, pf.s1.y);
            v[2] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
            v[3] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
            r[0] = Sp32{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
          }
          pc_apply<NW, 1, true>(a, S, Hs, tile * per, own, loc, val, jj, r, z);
          if (val[0]) {
            stf4(st.r, i, r[0]);
            own_st<P>(st.z, a.halo_z, i, z[0]);
            v[1] += double(rdotf(r[0], z[0]));
          }
          __syncthreads();
        }
        v2_publish<4>(v, a.partials, parity, sh);
        if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      }
      double tr[4];
      v2_total<4>(a.partials, parity, tr, sh);
      parity ^= 1;
      nru++;
      mu_true = tr[0];
      if (mu_true < a.tol2 * bnorm2) {
        status = QED3_OK;
        break;
      }
      if (iter >= a.maxiter || !isfinite(mu_true) || !(tr[1] > 0.0)) {
        status = QED3_ERR_NOCONV;
        break;
      }
      beta = tr[1] / rho;
      a_z = make_double2(1.0 - beta * tr[2] / tr[1], -beta * tr[3] / tr[1]);
      rho = tr[1];
      mu_max = mu_true;
    }
  finish:
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
// Pipelined preconditioned CG: ONE grid barrier per iteration
// ---------------------------------------------------------------------------
// Ghysels & Vanroose's pipelined PCG (u = N r, w = A u, s = A p, q = N s,
// z = A q, A = D^dag D + s):
//   gam = <r,u>, delta = <w,u>;  m = N w;  n = A m
//   beta = gam / gam_old, alpha = gam / (delta - beta gam / alpha_old)
//   z = n + beta z, q = m + beta q, s = w + beta s, p = u + beta p,
//   x += alpha p, r -= alpha s, u -= alpha q, w -= alpha z.
// The dots and m = N w (block-local) need no neighbour data, and A m is
// applied as a two-hop stencil from ONE gathered field,
//   (D m)_y = diag_y m_y + sum_k H_{y,k} m_{nbr(y,k)}   (y = i and its neighbours),
//   n_i = diag_i (D m)_i + sum_k Hd_{i,k} (D m)_{nbr(i,k)} + s m_i,
// so each iteration is [dots, m = N w, publish m | barrier | totals, n = A m,
// updates].  A residual replacement (FP64 reliable update, three barriers as
// in the other solvers) recomputes r = b - A x, u, w and s = A p, q = N s,
// z = A q, m = N w, n = A m exactly (two more barriers) and takes that step
// with a direct line search along p' = u + beta p: alpha = <r,p'> / <p',A p'>
// (in a CPU model of this recurrence in FP32 with FP64 replacements the
// iteration counts equal those of the two-barrier PCG at n = 16, 32, 64).

__device__ __forceinline__ Sp32 blk_mul(const float4& r0, const float4& r1, const Sp32& y) {
  Sp32 o;
  o.s0 = cfmaf(lo2(r0), y.s0, make_float2(0.f, 0.f));
  o.s0 = cfmaf(hi2(r0), y.s1, o.s0);
  o.s1 = cfmaf(lo2(r1), y.s0, make_float2(0.f, 0.f));
  o.s1 = cfmaf(hi2(r1), y.s1, o.s1);
  return o;
}

// n_i = (D^dag D + sig) m at owned site i from the gathered field `halo`.
// Every thread of the block calls it (two __syncthreads): each owned site
// computes (D m)_i from its own hop blocks (shared memory) and its three
// gathered neighbours and posts it to SDm; (D m)_j of an in-block neighbour
// is then read from SDm, that of a neighbour owned by another block is
// recomputed here from the gathered field (nb2[(3k+q) * per + lc] =
// nbr(nbr(i,k), q)) and that neighbour's hop blocks.
template <int P, bool TRAIL>
__device__ __forceinline__ Sp32 two_hop(bool ok, int i, int lc, int blk0, int per, int Ns, const int (&jj)[3],
                                        const int* nb2, const M32* __restrict__ H32,
                                        const float* __restrict__ diag32, const float4* HsD, const float4* HsDd,
                                        float4* SDm, float dg, float sig, const Sp32& self, const void* halo) {
  const Sp32 zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  Sp32 mn[3] = {zero, zero, zero};
  Sp32 dj[3] = {zero, zero, zero};  // (D m)_j of neighbours owned by other blocks
  Sp32 di = zero;
  if (ok) {
    // one round of loads: the three neighbours, and for neighbours owned by
    // another block their neighbours and hop blocks as well
#pragma unroll
    for (int k = 0; k < 3; k++) mn[k] = hl32<P>(halo, jj[k]);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int j = jj[k];
      if (unsigned(j - blk0) >= unsigned(per)) {
        Sp32 acc = zero;
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const float4* hm = reinterpret_cast<const float4*>(H32 + size_t(q) * Ns + j);
          acc = sp_add(acc, blk_mul(__ldg(hm), __ldg(hm + 1), hl32<P>(halo, nb2[(3 * k + q) * per + lc])), 1.f);
        }
        dj[k] = sp_add(acc, mn[k], __ldg(diag32 + j));
      }
    }
    di = sp_add(zero, self, dg);
#pragma unroll
    for (int k = 0; k < 3; k++)
      di = sp_add(di, blk_mul(HsD[(2 * k) * per + lc], HsD[(2 * k + 1) * per + lc], mn[k]), 1.f);
  }
  SDm[lc] = sp2f4(di);
  __syncthreads();
  Sp32 o = zero;
  if (ok) {
    o = sp_add(sp_add(zero, di, dg), self, sig);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int l = jj[k] - blk0;
      const Sp32 d = (unsigned(l) < unsigned(per)) ? f42sp(SDm[l]) : dj[k];
      o = sp_add(o, blk_mul(HsDd[(2 * k) * per + lc], HsDd[(2 * k + 1) * per + lc], d), 1.f);
    }
  }
  if (TRAIL) __syncthreads();  // SDm is read before a following call overwrites it
  return o;
}

// the recurrences of one pipelined step (z, q, s and the solution increment
// in the thread's shared slots)
__device__ __forceinline__ void ppcg_step(double alpha, double beta, const Sp32& n, const Sp32& m, Sp32& r, Sp32& u,
                                          Sp32& w, Sp32& p, float4* SZ, float4* SQ, float4* SS, float4* SX, int lc) {
  const float al = float(alpha), bt = float(beta);
  const Sp32 zz = sp_add(n, f42sp(SZ[lc]), bt);
  const Sp32 q = sp_add(m, f42sp(SQ[lc]), bt);
  const Sp32 s = sp_add(w, f42sp(SS[lc]), bt);
  p = sp_add(u, p, bt);
  SZ[lc] = sp2f4(zz);
  SQ[lc] = sp2f4(q);
  SS[lc] = sp2f4(s);
  SX[lc] = sp2f4(sp_add(f42sp(SX[lc]), p, al));
  r = sp_add(r, s, -al);
  u = sp_add(u, q, -al);
  w = sp_add(w, zz, -al);
}

// Phases of k_ppcg around its single preconditioner application (one inlined
// copy: five copies of the 7-word preconditioner spilled to local memory).
enum PpcgPhase { PH_INIT = 0, PH_MAIN = 1, PH_R2 = 2, PH_R3A = 3, PH_R3B = 4 };

template <int P, int NW>
__global__ void __launch_bounds__(576, 1) k_ppcg(PcgArgs a) {
  extern __shared__ float4 S[];
  __shared__ double sh[32 * 4 + 64 + 8];
  const int Ns = a.Ns, per = a.per;
  const int blk0 = blockIdx.x * per;
  float4* HsD = S + NW * per;
  float4* HsDd = HsD + 6 * per;
  int* nb2 = reinterpret_cast<int*>(HsDd + 6 * per);
  float4* SDm = reinterpret_cast<float4*>(nb2 + 9 * per);  // (D m) of the owned sites
  // thread-private slots (each thread touches only its own entry): the
  // recurrence vectors z, q, s and the fp32 solution increment live in shared
  // memory to keep the registers for the preconditioner
  float4* SZ = SDm + per;
  float4* SQ = SZ + per;
  float4* SS = SQ + per;
  float4* SX = SS + per;
  const int lc = threadIdx.x;  // one site per thread
  const int i = blk0 + lc;
  const bool ok = i < Ns;
  const int own[1] = {i}, loc[1] = {lc};
  const bool val[1] = {ok};
  int jj[1][3] = {{0, 0, 0}};
  float dg = 0.f;
  const Sp32 z32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  const float4 zf = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 6; q++) {
    HsD[q * per + lc] = ok ? __ldg(reinterpret_cast<const float4*>(a.H32 + size_t(q >> 1) * Ns + i) + (q & 1)) : zf;
    HsDd[q * per + lc] = ok ? __ldg(reinterpret_cast<const float4*>(a.Hd32 + size_t(q >> 1) * Ns + i) + (q & 1)) : zf;
  }
  if (ok) {
    dg = __ldg(a.diag32 + i);
#pragma unroll
    for (int k = 0; k < 3; k++) jj[0][k] = __ldg(a.nbr + k * Ns + i);
  }
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int q = 0; q < 3; q++) nb2[(3 * k + q) * per + lc] = ok ? __ldg(a.nbr + q * Ns + jj[0][k]) : 0;
  SZ[lc] = zf;
  SQ[lc] = zf;
  SS[lc] = zf;
  SX[lc] = zf;
  const float sig = float(a.shift);
  // A2(x, halo): (D^dag D + s) x from the gathered copy; the next write of SDm
  // is behind a grid barrier.  A2T: another A2 follows directly.
  const M32* const H32g = a.H32;
  const float* const dg32g = a.diag32;
#define A2(x, halo) two_hop<P, false>(ok, i, lc, blk0, per, Ns, jj[0], nb2, H32g, dg32g, HsD, HsDd, SDm, dg, sig, x, halo)
#define A2T(x, halo) two_hop<P, true>(ok, i, lc, blk0, per, Ns, jj[0], nb2, H32g, dg32g, HsD, HsDd, SDm, dg, sig, x, halo)

  Sp32 r = z32, u = z32, w = z32, p = z32;
  if (ok) {
    const Sp64 bi = ld64(a.b, i);
    r = Sp32{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
  }
  unsigned int epoch = 0;
  int parity = 0;
  double bnorm2 = 0.0, mu_true = 0.0, mu_max = 0.0, gam_old = 0.0, al_old = 0.0, ru_part = 0.0;
  int iter = 0, nru = 0, status = QED3_ERR_NOCONV;
  bool first = true;
  int phase = PH_INIT;
  while (true) {
    // ---- the single preconditioner application: u = N r (INIT, R2), m = N w (MAIN,
    //      R3B), q = N s (R3A) ----------------------------------------------------------
    Sp32 pin[1], pout[1];
    pin[0] = (phase == PH_INIT || phase == PH_R2) ? r : (phase == PH_R3A ? f42sp(SS[lc]) : w);
    pc_apply<NW, 1, true>(a, S, HsD, blk0, own, loc, val, jj, pin, pout);
    if (phase == PH_INIT) {
      u = pout[0];
      double v1[1] = {0.0};
      if (ok) {
        v1[0] = n2(ld64(a.b, i));
        hs32<P>(a.halo_u, i, u);
      }
      v2_publish<1>(v1, a.partials, parity, sh);
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      double tot[1];
      v2_total<1>(a.partials, parity, tot, sh);
      parity ^= 1;
      bnorm2 = tot[0];
      mu_true = mu_max = bnorm2;
      if (bnorm2 == 0.0) {
        status = QED3_OK;
        break;
      }
      w = A2(u, a.halo_u);
      phase = PH_MAIN;
      continue;
    }
    if (phase == PH_MAIN) {
      // ---- dots of (r, u, w), publish m = N w | barrier | totals ------------------------
      const Sp32 m = pout[0];
      float v[3] = {0.f, 0.f, 0.f};
      if (ok) {
        v[0] = rdotf(r, u);
        v[1] = rdotf(w, u);
        v[2] = n2f(r);
        hs32<P>(a.halo_z, i, m);
      }
      v2_publish_f<3>(v, a.partials, parity, sh);
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      double t3[3];
      v2_total<3>(a.partials, parity, t3, sh);
      parity ^= 1;
      const double gam = t3[0], dl = t3[1], mu = t3[2];
      mu_max = fmax(mu_max, mu);
      const bool want = !first && (!isfinite(mu) || !(gam > 0.0) || mu < a.tol2 * bnorm2 || iter >= a.maxiter ||
                                   mu < a.delta2 * mu_max);
      if (!want) {
        const double beta = first ? 0.0 : gam / gam_old;
        const double alpha = first ? gam / dl : gam / (dl - beta * gam / al_old);
        const Sp32 n = A2(m, a.halo_z);
        ppcg_step(alpha, beta, n, m, r, u, w, p, SZ, SQ, SS, SX, lc);
        gam_old = gam;
        al_old = alpha;
        first = false;
        iter++;
        continue;
      }
      // ---- residual replacement: R0 fold and publish x ------------------------------------
      Sp64 xh{make_double2(0, 0), make_double2(0, 0)};
      if (ok) {
        const Sp32 xl = f42sp(SX[lc]);
        xh = hl64(a.x, i);
        xh.s0 = make_double2(xh.s0.x + xl.s0.x, xh.s0.y + xl.s0.y);
        xh.s1 = make_double2(xh.s1.x + xl.s1.x, xh.s1.y + xl.s1.y);
        hs64(a.x, i, xh);
      }
      SX[lc] = zf;
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R1: t64 = D x ------------------------------------------------------------------
      if (ok) hs64(a.t64, i, stencil64(i, Ns, jj[0], a.H, a.diag, xh, a.x));
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      // ---- R2 (first half): r = b - D^dag t64 - s x in FP64 --------------------------------
      ru_part = 0.0;
      if (ok) {
        const Sp64 self = hl64(a.t64, i);
        const Sp64 qd = stencil64(i, Ns, jj[0], a.Hd, a.diag, self, a.t64);
        const Sp64 bi = ld64(a.b, i);
        Sp64 rt;
        rt.s0 = csub(bi.s0, cadd(qd.s0, cscale(a.shift, xh.s0)));
        rt.s1 = csub(bi.s1, cadd(qd.s1, cscale(a.shift, xh.s1)));
        ru_part = n2(rt);
        r = Sp32{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
      }
      phase = PH_R2;  // u = N r next
      continue;
    }
    if (phase == PH_R2) {
      // ---- R2 (second half): publish u = N r and p | barrier | certificate ----------------
      u = pout[0];
      if (ok) {
        hs32<P>(a.halo_u, i, u);
        hs32<P>(a.halo_p, i, p);
      }
      double vv[1] = {ru_part};
      v2_publish<1>(vv, a.partials, parity, sh);
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      double tr[1];
      v2_total<1>(a.partials, parity, tr, sh);
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
      mu_max = mu_true;
      // ---- R3: w = A u, s = A p (q = N s, m = N w follow) --------------------------------
      w = A2T(u, a.halo_u);
      SS[lc] = sp2f4(A2T(p, a.halo_p));
      phase = PH_R3A;
      continue;
    }
    if (phase == PH_R3A) {
      SQ[lc] = sp2f4(pout[0]);
      phase = PH_R3B;
      continue;
    }
    // ---- PH_R3B: publish q, m; line-search dots | barrier | z = A q, n = A m, step ------
    {
      const Sp32 m = pout[0];
      const Sp32 q = f42sp(SQ[lc]), sv = f42sp(SS[lc]);
      float v5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (ok) {
        hs32<P>(a.halo_q, i, q);
        hs32<P>(a.halo_z, i, m);
        v5[0] = rdotf(r, u);
        v5[1] = rdotf(r, p);
        v5[2] = rdotf(u, w);
        v5[3] = rdotf(u, sv) + rdotf(p, w);
        v5[4] = rdotf(p, sv);
      }
      v2_publish_f<5, 8>(v5, a.partials, parity, sh);
      if (!grid_sync2(a.bar, epoch, a.spin_limit)) goto timeout;
      double t5[5];
      v2_total<5, 8>(a.partials, parity, t5, sh);
      parity ^= 1;
      const double gam = t5[0];
      const double beta = gam / gam_old;
      const double rp = gam + beta * t5[1];
      const double pap = t5[2] + beta * t5[3] + beta * beta * t5[4];
      const double alpha = rp / pap;
      SZ[lc] = sp2f4(A2T(q, a.halo_q));
      const Sp32 n = A2(m, a.halo_z);
      ppcg_step(alpha, beta, n, m, r, u, w, p, SZ, SQ, SS, SX, lc);
      gam_old = gam;
      al_old = alpha;
      first = false;
      iter++;
      phase = PH_MAIN;
    }
  }
  // finish: x was published at the last residual replacement (or is zero)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[0] = mu_true;
    a.scal[1] = bnorm2;
    a.scal[2] = iter;
    a.scal[3] = nru;
    a.scal[4] = status;
    a.scal[5] = 0;
  }
  return;
timeout:
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[4] = QED3_ERR_TIMEOUT;
    a.scal[5] = 0;
  }
}
#undef A2
#undef A2T

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int P, int NW, int SPT>
static const void* pcg_fn() {
  return (const void*)k_pcg<P, NW, SPT>;
}

static const void* pcg_kernel(int prec, int nw, int spt) {
  if (prec == QED3_PREC_F32) {
    if (nw == 7) return spt == 1 ? pcg_fn<P32, 7, 1>() : pcg_fn<P32, 7, 2>();
    return spt == 1 ? pcg_fn<P32, 3, 1>() : pcg_fn<P32, 3, 2>();
  }
  if (nw == 7) return spt == 1 ? pcg_fn<PBF16, 7, 1>() : pcg_fn<PBF16, 7, 2>();
  return spt == 1 ? pcg_fn<PBF16, 3, 1>() : pcg_fn<PBF16, 3, 2>();
}

// The preconditioner's block partition: one block per SM while a block fits
// the register-resident solver (<= 1152 sites), else tiles of <= 512 sites,
// k per SM, for the streaming solver (512 threads: four warps per SM
// sub-partition, so 128 registers per thread).  Training and solver share it.
int pcg_block_sites(int Ns, int sm_count) {
  const long long per_sm = (Ns + sm_count - 1) / sm_count;
  if (per_sm <= 576) return int((per_sm + 31) / 32 * 32);
  if (per_sm <= 1152) return int((per_sm + 63) / 64 * 64);
  const long long k = (per_sm + 511) / 512;
  const long long per = (Ns + k * sm_count - 1) / (k * sm_count);
  return int((per + 31) / 32 * 32);
}

static const void* ppcg_kernel(int prec, int nw) {
  if (prec == QED3_PREC_F32) return nw == 7 ? (const void*)k_ppcg<P32, 7> : (const void*)k_ppcg<P32, 3>;
  return nw == 7 ? (const void*)k_ppcg<PBF16, 7> : (const void*)k_ppcg<PBF16, 3>;
}

// The pipelined kernel: one site per thread, per <= 576; shared memory holds the
// preconditioner fields, the owned hop blocks of D and D^dag and the two-hop ids.
static bool ppcg_plan(int prec, int nw, int Ns, int per, int sm_count, int* grid, size_t* smem) {
  if (per % 32 || per > 576) return false;
  const void* fn = ppcg_kernel(prec, nw);
  const size_t sm = size_t(nw + 17) * per * sizeof(float4) + size_t(9) * per * sizeof(int);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, per, sm) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int G = (Ns + per - 1) / per;
  if (per_sm < 1 || G > per_sm * sm_count) return false;
  *grid = G;
  *smem = sm;
  return true;
}

bool pcg_plan(int prec, int nw, int Ns, int per, int sm_count, int* grid, int* threads, int* spt, size_t* smem) {
  for (int s : {1, 2}) {
    if (per % (32 * s)) continue;
    const int T = per / s;
    if (T > 576) continue;
    const void* fn = pcg_kernel(prec, nw, s);
    const size_t sm = size_t(nw + 1 + (s == 1 ? 12 : 0)) * per * sizeof(float4);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, sm) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    const int G = (Ns + per - 1) / per;
    if (per_sm < 1 || G > per_sm * sm_count) continue;
    *grid = G;
    *threads = T;
    *spt = s;
    *smem = sm;
    return true;
  }
  return false;
}

static const void* pcgs_kernel(int prec, int nw) {
  if (prec == QED3_PREC_F32) return nw == 7 ? (const void*)k_pcgs<P32, 7> : (const void*)k_pcgs<P32, 3>;
  return nw == 7 ? (const void*)k_pcgs<PBF16, 7> : (const void*)k_pcgs<PBF16, 3>;
}

// The streaming kernel: per threads (one site of the current tile each), the
// preconditioner fields and the tile's hop blocks in shared memory, one block
// per SM.
static bool pcgs_plan(int prec, int nw, int Ns, int per, int sm_count, int* grid, size_t* smem) {
  if (per % 32 || per > 512) return false;
  const void* fn = pcgs_kernel(prec, nw);
  const size_t sm = size_t(nw + 6) * per * sizeof(float4);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, per, sm) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (per_sm < 1) return false;
  const int tiles = (Ns + per - 1) / per;
  *grid = std::min(tiles, sm_count);
  *smem = sm;
  return true;
}

int pcg_solve(qed3_dirac_s* d, qed3_lpc_s* L, double* x, const double* b, const qed3_solve_params* prm,
              qed3_solve_report* rep, cudaStream_t st) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set (call qed3_dirac_set_links)");
  if (L->Ns != d->Ns) return fail(QED3_ERR_ARG, "preconditioner and operator live on different lattices");
  int rc = ensure_work(d);
  if (rc) return rc;
  SolverWork& w = d->work;
  const int prec = prm ? prm->precision : QED3_PREC_F32;
  if (prec != QED3_PREC_F32 && prec != QED3_PREC_BF16)
    return fail(QED3_ERR_ARG, "preconditioned CG runs in mixed precision (QED3_PREC_F32 or QED3_PREC_BF16)");
  const double tol = prm && prm->tol > 0 ? prm->tol : 1e-10;
  const double delta = prm && prm->delta > 0 ? prm->delta : 0.1;
  const int maxiter = prm && prm->maxiter > 0 ? prm->maxiter : 100000;
  const double shift = prm ? prm->shift : 0.0;
  LpcWordCoef co;
  if ((rc = lpc_word_coef_cached(L, &co))) return rc;
  const bool flexible = prm && (prm->flags & QED3_SOLVE_FLEXIBLE);
  // the pipelined recurrence is FP32-only: with BF16 gathered copies its
  // auxiliary vectors drift apart (measured: 43,000 instead of 240 iterations)
  const bool want_pipe = prm && (prm->flags & QED3_SOLVE_PIPELINED) && !flexible && prec == QED3_PREC_F32;
  int grid = 0, threads = 0, spt = 0;
  size_t smem = 0;
  const bool pipelined = want_pipe && ppcg_plan(prec, co.nwords, d->Ns, L->per, d->sm_count, &grid, &smem);
  bool streaming = false;
  if (!pipelined && !pcg_plan(prec, co.nwords, d->Ns, L->per, d->sm_count, &grid, &threads, &spt, &smem)) {
    if (flexible) return fail(QED3_ERR_ARG, "flexible preconditioned CG needs the register-resident solver (n <= ~93)");
    if (!pcgs_plan(prec, co.nwords, d->Ns, L->per, d->sm_count, &grid, &smem))
      return fail(QED3_ERR_ARG, "no preconditioned solver layout for this lattice and block size");
    streaming = true;
  }
  if ((rc = field_import_unit(d, w.b, b, w.partials, w.scal + 6, st))) return rc;
  if (pipelined) QED3_CUDA_TRY(cudaMemsetAsync(w.xhi, 0, size_t(d->Ns) * 4 * sizeof(double), st));
  QED3_CUDA_TRY(cudaMemsetAsync(w.bar2, 0, sizeof(GridBar2), st));
  PcgArgs a{};
  a.Ns = d->Ns;
  a.per = L->per;
  a.nbr = d->lat->dev.nbr;
  a.H = d->H;
  a.Hd = d->Hd;
  a.diag = d->diag;
  a.H32 = d->H32;
  a.Hd32 = d->Hd32;
  a.diag32 = d->diag32;
  a.b = w.b;
  a.x = w.xhi;
  a.t64 = w.t64;
  a.halo_z = w.r;
  a.halo_t = w.t;
  a.partials = w.partials;
  a.bar = w.bar2;
  a.scal = w.scal;
  a.tol2 = tol * tol;
  a.delta2 = delta * delta;
  a.shift = shift;
  a.maxiter = maxiter;
  a.flexible = (prm && (prm->flags & QED3_SOLVE_FLEXIBLE)) ? 1 : 0;
  a.spin_limit = 4000000LL;
  a.pc = co;
  a.halo_u = w.t;
  a.halo_p = w.p;
  a.halo_q = w.xlo;
  void* kargs[] = {&a};
  QED3_CUDA_TRY(cudaEventRecord(w.e0, st));
  PcgsState ss{reinterpret_cast<float4*>(w.tg), reinterpret_cast<float4*>(w.p), reinterpret_cast<float4*>(w.rhi),
               reinterpret_cast<float4*>(w.rg), reinterpret_cast<float4*>(w.xlo)};
  void* sargs[] = {&a, &ss};
  if (pipelined)
    QED3_CUDA_TRY(cudaLaunchCooperativeKernel(ppcg_kernel(prec, co.nwords), dim3(grid), dim3(L->per), kargs, smem, st));
  else if (streaming)
    QED3_CUDA_TRY(cudaLaunchCooperativeKernel(pcgs_kernel(prec, co.nwords), dim3(grid), dim3(L->per), sargs, smem, st));
  else
    QED3_CUDA_TRY(
        cudaLaunchCooperativeKernel(pcg_kernel(prec, co.nwords, spt), dim3(grid), dim3(threads), kargs, smem, st));
  QED3_CUDA_TRY(cudaEventRecord(w.e1, st));
  return cg_finish(d, x, rep, st);
}

}  // namespace qed3
