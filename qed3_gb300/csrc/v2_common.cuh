// Device helpers shared by the register-resident persistent solvers
// (solver_v2.cu, pcg.cu): reductions riding on the grid barrier, halo
// loads/stores through L2, and the one-site stencils.
#pragma once

#include <cuda_bf16.h>

#include "device.cuh"

namespace qed3 {

template <int NV>
__device__ __forceinline__ void v2_publish(double (&v)[NV], double* part, int parity, double* sh) {
  block_sum<NV>(v, sh);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) __stcg(part + (size_t(parity) * gridDim.x + blockIdx.x) * 4 + q, v[q]);
}

// Global totals: lane l of warp 0 loads the partials of blocks l, l+32, ...
// all at once (one L2 round trip instead of one per block stride), then FP64
// sums in a fixed order (deterministic), broadcast through shared memory.
// W: doubles per block slot in `part` (>= NV)
template <int NV, int W = 4>
__device__ __forceinline__ void v2_total(const double* part, int parity, double (&out)[NV], double* sh) {
  static_assert(NV <= W, "slot too small");
  if (threadIdx.x < 32) {
    const int G = gridDim.x;
    const double* base = part + size_t(parity) * G * W;
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = 0.0;
    // fixed trip count: the loads of all strides are independent and issue together
#pragma unroll
    for (int c = 0; c < 5; c++) {
      const int bI = threadIdx.x + 32 * c;
#pragma unroll
      for (int q = 0; q < NV; q++) acc[q] += bI < G ? __ldcg(base + size_t(bI) * W + q) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < NV; q++) {
      for (int bI = threadIdx.x + 160; bI < G; bI += 32) acc[q] += __ldcg(base + size_t(bI) * W + q);
      acc[q] = warp_sum(acc[q]);
    }
    if (threadIdx.x == 0)
#pragma unroll
      for (int q = 0; q < NV; q++) sh[64 + q] = acc[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; q++) out[q] = sh[64 + q];
  __syncthreads();
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block partial of NV fp32 values (the inner iteration's |t|^2, |r|^2, <r,z>):
// fp32 warp and cross-warp sums, one conversion, the FP64 partial stored for
// the global FP64 accumulation in v2_total.  FP64 arithmetic stays off the
// per-thread path: on GB300 a dependent DADD costs ~2.5x an FADD, a 64-bit
// shuffle ~2x, and an f32<->f64 conversion ~4x.
template <int NV, int W = 4>
__device__ __forceinline__ void v2_publish_f(float (&v)[NV], double* part, int parity, double* sh) {
  static_assert(NV <= W, "slot too small");
  float* shf = reinterpret_cast<float*>(sh);  // 32*NV floats, below the totals' slots
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum_f(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) shf[q * 32 + warp] = v[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      float t = lane < nw ? shf[q * 32 + lane] : 0.f;
      t = warp_sum_f(t);
      if (lane == 0) __stcg(part + (size_t(parity) * gridDim.x + blockIdx.x) * W + q, double(t));
    }
  }
}

// halo access (L2, bypassing L1: written by other SMs in the previous phase)
__device__ __forceinline__ Sp64 hl64(const S64* f, int i) {
  const double2* p = reinterpret_cast<const double2*>(f + i);
  return {__ldcg(p), __ldcg(p + 1)};
}
__device__ __forceinline__ void hs64(S64* f, int i, Sp64 v) {
  double2* p = reinterpret_cast<double2*>(f + i);
  __stcg(p, v.s0);
  __stcg(p + 1, v.s1);
}
template <int P>
__device__ __forceinline__ Sp32 hl32(const void* f, int i) {
  if constexpr (P == PBF16) {
    const uint2 v = __ldcg(reinterpret_cast<const uint2*>(f) + i);
    __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&v.x);
    __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&v.y);
    return {__bfloat1622float2(a), __bfloat1622float2(b)};
  } else {
    const float4 v = __ldcg(reinterpret_cast<const float4*>(f) + i);
    return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
  }
}
template <int P>
__device__ __forceinline__ void hs32(void* f, int i, Sp32 v) {
  if constexpr (P == PBF16) {
    __nv_bfloat162 a = __float22bfloat162_rn(v.s0);
    __nv_bfloat162 b = __float22bfloat162_rn(v.s1);
    uint2 o;
    o.x = *reinterpret_cast<uint32_t*>(&a);
    o.y = *reinterpret_cast<uint32_t*>(&b);
    __stcg(reinterpret_cast<uint2*>(f) + i, o);
  } else {
    __stcg(reinterpret_cast<float4*>(f) + i, make_float4(v.s0.x, v.s0.y, v.s1.x, v.s1.y));
  }
}

__device__ __forceinline__ double n2(const Sp64& a) {
  return a.s0.x * a.s0.x + a.s0.y * a.s0.y + a.s1.x * a.s1.x + a.s1.y * a.s1.y;
}
__device__ __forceinline__ float n2f(const Sp32& a) {
  return a.s0.x * a.s0.x + a.s0.y * a.s0.y + a.s1.x * a.s1.x + a.s1.y * a.s1.y;
}

// own-site value o = diag * self + sum_k H_k * halo[nbr_k]   (fp64)
__device__ __forceinline__ Sp64 stencil64(int i, int Ns, const int (&jj)[3], const M64* __restrict__ H,
                                          const double* __restrict__ diag, const Sp64& self, const S64* halo) {
  const double dg = __ldg(diag + i);
  Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
  const Sp64 b0 = hl64(halo, jj[0]), b1 = hl64(halo, jj[1]), b2 = hl64(halo, jj[2]);
  const Sp64 bs[3] = {b0, b1, b2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double2* m = reinterpret_cast<const double2*>(H + size_t(k) * Ns + i);
    const double2 h00 = __ldg(m), h01 = __ldg(m + 1), h10 = __ldg(m + 2), h11 = __ldg(m + 3);
    o.s0 = cfma(h00, bs[k].s0, o.s0);
    o.s0 = cfma(h01, bs[k].s1, o.s0);
    o.s1 = cfma(h10, bs[k].s0, o.s1);
    o.s1 = cfma(h11, bs[k].s1, o.s1);
  }
  return o;
}

template <int P>
__device__ __forceinline__ Sp32 stencil32(int i, int Ns, const int (&jj)[3], const M32* __restrict__ H,
                                          const float* __restrict__ diag, const Sp32& self, const void* halo) {
  const float dg = __ldg(diag + i);
  Sp32 o{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
  const Sp32 b0 = hl32<P>(halo, jj[0]), b1 = hl32<P>(halo, jj[1]), b2 = hl32<P>(halo, jj[2]);
  const Sp32 bs[3] = {b0, b1, b2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float4* m = reinterpret_cast<const float4*>(H + size_t(k) * Ns + i);
    const float4 r0 = __ldg(m), r1 = __ldg(m + 1);
    o.s0 = cfmaf(make_float2(r0.x, r0.y), bs[k].s0, o.s0);
    o.s0 = cfmaf(make_float2(r0.z, r0.w), bs[k].s1, o.s0);
    o.s1 = cfmaf(make_float2(r1.x, r1.y), bs[k].s0, o.s1);
    o.s1 = cfmaf(make_float2(r1.z, r1.w), bs[k].s1, o.s1);
  }
  return o;
}

}  // namespace qed3
