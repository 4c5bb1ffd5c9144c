// Device-side types and helpers shared by the sm_103a kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace qed3 {

// ---------------------------------------------------------------------------
// Field layouts (one two-spinor per site, sites in space-filling-curve order)
//   F64 : 32 B  {double2 s0, s1}
//   F32 : 16 B  float4 (s0.re, s0.im, s1.re, s1.im)
//   BF16:  8 B  four bf16 in a uint2, converted to fp32 on load
// Hop matrices (one 2x2 complex block per directed hop, SoA over the 3 slots)
//   M64 : 64 B  {h00, h01, h10, h11} double2
//   M32 : 32 B  float4 row0 (h00, h01), float4 row1 (h10, h11)
// ---------------------------------------------------------------------------
struct __align__(16) S64 {
  double2 s0, s1;
};
struct __align__(16) M64 {
  double2 h00, h01, h10, h11;
};
struct __align__(16) M32 {
  float4 r0, r1;
};

enum Prec { P64 = 0, P32 = 1, PBF16 = 2 };

// ---- complex arithmetic ----------------------------------------------------
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc + a*b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
__device__ __forceinline__ float2 cfmaf(float2 a, float2 b, float2 acc) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
  return acc;
}

// ---- field access by precision ---------------------------------------------
struct Sp32 {
  float2 s0, s1;
};
struct Sp64 {
  double2 s0, s1;
};

__device__ __forceinline__ Sp64 ld64(const S64* f, int i) {
  const S64 v = f[i];
  return {v.s0, v.s1};
}
__device__ __forceinline__ void st64(S64* f, int i, Sp64 v) { f[i] = S64{v.s0, v.s1}; }

__device__ __forceinline__ Sp32 ld32(const float4* f, int i) {
  const float4 v = f[i];
  return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ void st32(float4* f, int i, Sp32 v) { f[i] = make_float4(v.s0.x, v.s0.y, v.s1.x, v.s1.y); }

__device__ __forceinline__ Sp32 ldbf(const uint2* f, int i) {
  const uint2 v = f[i];
  __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&v.x);
  __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&v.y);
  return {__bfloat1622float2(a), __bfloat1622float2(b)};
}
__device__ __forceinline__ void stbf(uint2* f, int i, Sp32 v) {
  __nv_bfloat162 a = __float22bfloat162_rn(v.s0);
  __nv_bfloat162 b = __float22bfloat162_rn(v.s1);
  uint2 o;
  o.x = *reinterpret_cast<uint32_t*>(&a);
  o.y = *reinterpret_cast<uint32_t*>(&b);
  f[i] = o;
}

// Generic low-precision field pointer: fp32 or bf16 storage.
template <int P>
struct LoField;
template <>
struct LoField<P32> {
  using T = float4;
  static __device__ __forceinline__ Sp32 ld(const T* f, int i) { return ld32(f, i); }
  static __device__ __forceinline__ void st(T* f, int i, Sp32 v) { st32(f, i, v); }
};
template <>
struct LoField<PBF16> {
  using T = uint2;
  static __device__ __forceinline__ Sp32 ld(const T* f, int i) { return ldbf(f, i); }
  static __device__ __forceinline__ void st(T* f, int i, Sp32 v) { stbf(f, i, v); }
};

// ---- one site of D or D^dagger ----------------------------------------------
// out = diag * in[i] + sum_k H[k][i] in[nbr[k][i]]
__device__ __forceinline__ Sp64 hop64(int i, int Ns, const int* __restrict__ nbr, const M64* __restrict__ H,
                                      const double* __restrict__ diag, const S64* __restrict__ in) {
  const int j0 = __ldg(nbr + i), j1 = __ldg(nbr + Ns + i), j2 = __ldg(nbr + 2 * Ns + i);
  const Sp64 a = ld64(in, i), b0 = ld64(in, j0), b1 = ld64(in, j1), b2 = ld64(in, j2);
  const double d = __ldg(diag + i);
  Sp64 o{cscale(d, a.s0), cscale(d, a.s1)};
  const M64 m0 = H[i], m1 = H[Ns + i], m2 = H[2 * Ns + i];
  o.s0 = cfma(m0.h00, b0.s0, o.s0);
  o.s0 = cfma(m0.h01, b0.s1, o.s0);
  o.s1 = cfma(m0.h10, b0.s0, o.s1);
  o.s1 = cfma(m0.h11, b0.s1, o.s1);
  o.s0 = cfma(m1.h00, b1.s0, o.s0);
  o.s0 = cfma(m1.h01, b1.s1, o.s0);
  o.s1 = cfma(m1.h10, b1.s0, o.s1);
  o.s1 = cfma(m1.h11, b1.s1, o.s1);
  o.s0 = cfma(m2.h00, b2.s0, o.s0);
  o.s0 = cfma(m2.h01, b2.s1, o.s0);
  o.s1 = cfma(m2.h10, b2.s0, o.s1);
  o.s1 = cfma(m2.h11, b2.s1, o.s1);
  return o;
}

template <int P>
__device__ __forceinline__ Sp32 hop32(int i, int Ns, const int* __restrict__ nbr, const M32* __restrict__ H,
                                      const float* __restrict__ diag, const typename LoField<P>::T* __restrict__ in) {
  const int j0 = __ldg(nbr + i), j1 = __ldg(nbr + Ns + i), j2 = __ldg(nbr + 2 * Ns + i);
  const Sp32 a = LoField<P>::ld(in, i), b0 = LoField<P>::ld(in, j0), b1 = LoField<P>::ld(in, j1),
             b2 = LoField<P>::ld(in, j2);
  const float d = __ldg(diag + i);
  Sp32 o{make_float2(d * a.s0.x, d * a.s0.y), make_float2(d * a.s1.x, d * a.s1.y)};
  const Sp32 bs[3] = {b0, b1, b2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const M32 m = H[k * Ns + i];
    o.s0 = cfmaf(make_float2(m.r0.x, m.r0.y), bs[k].s0, o.s0);
    o.s0 = cfmaf(make_float2(m.r0.z, m.r0.w), bs[k].s1, o.s0);
    o.s1 = cfmaf(make_float2(m.r1.x, m.r1.y), bs[k].s0, o.s1);
    o.s1 = cfmaf(make_float2(m.r1.z, m.r1.w), bs[k].s1, o.s1);
  }
  return o;
}

// diag * self + sum_k H[k][i] halo[nbr[k][i]]: the own value comes from the
// fp32 state, the neighbours from the gathered copy (fp32 or bf16).
template <int P>
__device__ __forceinline__ Sp32 hop32_self(int i, int Ns, const int* __restrict__ nbr, const M32* __restrict__ H,
                                           const float* __restrict__ diag, const Sp32& self,
                                           const typename LoField<P>::T* halo) {
  const int j0 = __ldg(nbr + i), j1 = __ldg(nbr + Ns + i), j2 = __ldg(nbr + 2 * Ns + i);
  const Sp32 bs[3] = {LoField<P>::ld(halo, j0), LoField<P>::ld(halo, j1), LoField<P>::ld(halo, j2)};
  const float d = __ldg(diag + i);
  Sp32 o{make_float2(d * self.s0.x, d * self.s0.y), make_float2(d * self.s1.x, d * self.s1.y)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const M32 m = H[k * Ns + i];
    o.s0 = cfmaf(make_float2(m.r0.x, m.r0.y), bs[k].s0, o.s0);
    o.s0 = cfmaf(make_float2(m.r0.z, m.r0.w), bs[k].s1, o.s0);
    o.s1 = cfmaf(make_float2(m.r1.x, m.r1.y), bs[k].s0, o.s1);
    o.s1 = cfmaf(make_float2(m.r1.z, m.r1.w), bs[k].s1, o.s1);
  }
  return o;
}

// ---- reductions ----------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV values; result valid in thread 0.  `sh` holds 32*NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) sh[q * 32 + warp] = v[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double t = lane < nw ? sh[q * 32 + lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

// ---- bounded grid barrier --------------------------------------------------------
// Used only by cooperative launches (all blocks co-resident).  Every wait is
// capped; on expiry the barrier sets `abort` and returns, and every block
// leaves the solver at its next check.  The state must be zeroed before each
// launch (stream-ordered memset).
struct GridBar {
  unsigned int count;
  unsigned int gen;
  int abort;
  int pad;
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile_int(const int* p) { return *(volatile const int*)p; }

// Returns true if the barrier completed, false if the solve must abort.
__device__ __forceinline__ bool grid_sync(GridBar* bar, unsigned int& gen, long long spin_limit) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    const unsigned int prev = atomicAdd(&bar->count, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      st_release(&bar->gen, gen + 1u);
    } else {
      long long spins = 0;
      while (ld_acquire(&bar->gen) == gen) {
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
    }
    if (ld_volatile_int(&bar->abort)) ok = 0;
    gen += 1u;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---- per-system step wait (dynamic batched schedule) ---------------------------
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits (one thread) until *epoch >= step, i.e. the system has completed the
// step before `step`, or until its state reads `done_state`.  Returns 0 when
// the step may start, 1 when the system is done, 2 when the wait ran out
// (after spin_limit polls it raises *abort) or another wait raised *abort.
__device__ __forceinline__ int wait_step(const int* epoch, int step, const volatile int* state, int done_state,
                                         int* abort, long long spin_limit) {
  long long spins = 0;
  while (true) {
    if (*state == done_state) return 1;
    if (ld_acquire_s32(epoch) >= step) return 0;
    if (ld_volatile_int(abort)) return 2;
    if (++spins > spin_limit) {
      atomicExch(abort, 1);
      return 2;
    }
    __nanosleep(32);
  }
}

// ---- grid barrier, monotonic form -------------------------------------------
// The arrival counter and the generation only grow within a launch (both are
// zeroed before it), so no reset sits on the critical path: the block whose
// acq_rel increment completes epoch * gridDim.x arrivals releases the new
// generation; the others acquire-poll it.  Counter, generation and abort flag
// sit on separate 128-byte lines.  Every wait is capped as in grid_sync.
struct __align__(128) GridBar2 {
  unsigned int count;
  unsigned int pad0[31];
  unsigned int gen;
  unsigned int pad1[31];
  int abort;
  int pad2[31];
};

__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ bool grid_sync2(GridBar2* bar, unsigned int& epoch, long long spin_limit) {
  __syncthreads();
  __shared__ int s_ok2;
  if (threadIdx.x == 0) {
    int ok = 1;
    epoch += 1u;
    const unsigned int target = epoch * gridDim.x;
    const unsigned int prev = atom_add_acq_rel(&bar->count, 1u);
    if (prev == target - 1u) {
      st_release(&bar->gen, epoch);
    } else {
      long long spins = 0;
      while (int(ld_acquire(&bar->gen) - epoch) < 0) {
        if ((spins & 63) == 63 && ld_volatile_int(&bar->abort)) {
          ok = 0;
          break;
        }
        if (++spins > spin_limit) {
          atomicExch(&bar->abort, 1);
          ok = 0;
          break;
        }
      }
    }
    s_ok2 = ok;
  }
  __syncthreads();
  return s_ok2 != 0;
}

}  // namespace qed3
