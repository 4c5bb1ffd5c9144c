// Tensor-core channel mixing of the learned preconditioner (tcgen05 + TMA).
//
// No counterpart in the reference.  The 16 -> 16 complex channel layer of the
// network, L(h) = W0 h + W1 Hd h + W2 Ho h, and its adjoint, written as real
// GEMMs over rows = (sample, site, spin):
//
//   mixing : out[row, n] = sum_k X[row, k] Wb[n, k]        M = rows (128-row tiles),
//            K = 3 tensors x 32 (re, im of 16 channels), N = 32 (re, im of 16 channels)
//   wgrad  : P[m, n] = sum_row X[row, m] G[row, n]          M = 96 (padded to 128),
//            N = 32, K = rows (split over CTAs, FP64 sum of the partials)
//
// BF16 operands in shared memory, FP32 accumulators in tensor memory
// (tcgen05.mma kind::f16, one elected thread), read back with tcgen05.ld.
// The mixing kernel stages activation tiles with 2-D TMA loads
// (cp.async.bulk.tensor) completing on an mbarrier, double buffered; the
// weight-gradient kernel transposes its tiles into the K-major layout with
// plain loads (K = rows there).  Shared-memory operand layout (both kernels):
// canonical K-major, no swizzle -- core matrices of 8 rows x 16 bytes, SBO =
// stride between 8-row groups, LBO = stride between 16-byte K chunks.
//
// Every wait on an mbarrier is bounded: on expiry the kernel sets *err, stops
// issuing work, waits (bounded) for what it has in flight, frees its tensor
// memory and returns.

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "device.cuh"
#include "handles.h"
#include "lpc_impl.h"
#include "qed3_internal.h"
#include "tc_impl.h"

namespace qed3 {

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of the given parity: true when it completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, long long limit) {
  for (long long i = 0; i < limit; i++) {
    if (mbar_test(b, parity)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {  // whole warp
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {  // whole warp
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: canonical K-major layout without swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor, kind::f16: D fp32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}
// byte offset of element (r, k) in a K-major no-swizzle operand with the given strides
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, uint32_t lbo, uint32_t sbo) {
  return uint32_t(r >> 3) * sbo + uint32_t(k >> 3) * lbo + uint32_t(r & 7) * 16u + uint32_t(k & 7) * 2u;
}

// ---------------------------------------------------------------------------
// mixing: out[row, 0:32] = sum_j X_j[row, 0:32] . Wb_j
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;                       // rows per tile (MMA M)
constexpr int kTcChunk = kTcRows * 16;             // one 16-byte K chunk of a tile: 2048 B
constexpr int kTcStage = 3 * 4 * kTcChunk;         // 3 tensors x 4 chunks: 24 KB
constexpr int kTcBBytes = 12 * 4 * 128;            // weights: 12 K chunks x 4 N groups x 128 B
constexpr uint32_t kTcIdesc = idesc_bf16(128, 32);
constexpr int kTcMixSmem = 2 * kTcStage + kTcBBytes + 1024;

struct TcMixArgs {
  int rows;
  int ntiles;
  const float2* W;  // layer weights [3][16][16] complex
  int adj;          // 1: adjoint layer (conjugate transpose, -W2)
  float* out;       // fp32 [rows][32]
  int* err;
  long long spin;
};

__global__ void __launch_bounds__(128) k_tc_mix(const __grid_constant__ CUtensorMap tm0,
                                                 const __grid_constant__ CUtensorMap tm1,
                                                 const __grid_constant__ CUtensorMap tm2, TcMixArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[2];
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tslot;
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* Asm = base;                   // [2 stages][3][4 chunks][2048]
  uint8_t* Bsm = base + 2 * kTcStage;    // [12 chunks][4 groups][128]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const CUtensorMap* maps[3] = {&tm0, &tm1, &tm2};

  // weights -> Wb[n][k] (bf16, K-major): n = 2 co + q, k = 32 j + 2 c + p
  for (int e = tid; e < 32 * 96; e += blockDim.x) {
    const int n = e / 96, k = e % 96;
    const int co = n >> 1, q = n & 1, j = k >> 5, c = (k & 31) >> 1, p = k & 1;
    float2 w;
    if (!a.adj) {
      w = a.W[(j * 16 + co) * 16 + c];
    } else {  // W'_j[co][c] = s_j conj(W_j[c][co]), s = (+, +, -)
      const float2 t = a.W[(j * 16 + c) * 16 + co];
      const float sg = (j == 2) ? -1.f : 1.f;
      w = make_float2(sg * t.x, -sg * t.y);
    }
    // (q, p): (0,0) Re w, (0,1) -Im w, (1,0) Im w, (1,1) Re w
    const float v = (q == p) ? w.x : (q == 0 ? -w.y : w.y);
    *reinterpret_cast<__nv_bfloat16*>(Bsm + kmaj_off(n, k, 512, 128)) = __float2bfloat16_rn(v);
  }
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&mma_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tslot, 32);
  fence_proxy_async();  // generic-proxy writes of Wb visible to the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;

  const int first = blockIdx.x;
  uint32_t ph_full[2] = {0, 0}, ph_mma = 0;
  bool issued[2] = {false, false};  // thread 0: a TMA into this stage not yet waited for
  bool mma_pending = false;         // thread 0: a commit not yet waited for
  bool bad = false;
  if (tid == 0 && first < a.ntiles) {
    mbar_arrive_expect_tx(&full[0], kTcStage);
    for (int j = 0; j < 3; j++)
      for (int kc = 0; kc < 4; kc++)
        tma_load_2d(Asm + (j * 4 + kc) * kTcChunk, maps[j], kc * 8, first * kTcRows, &full[0]);
    issued[0] = true;
  }
  int it = 0;
  for (int tile = first; tile < a.ntiles; tile += gridDim.x, it++) {
    const int s = it & 1;
    const int next = tile + gridDim.x;
    if (tid == 0 && next < a.ntiles) {  // prefetch into the other stage (its MMAs completed last tile)
      mbar_arrive_expect_tx(&full[s ^ 1], kTcStage);
      for (int j = 0; j < 3; j++)
        for (int kc = 0; kc < 4; kc++)
          tma_load_2d(Asm + (s ^ 1) * kTcStage + (j * 4 + kc) * kTcChunk, maps[j], kc * 8, next * kTcRows,
                      &full[s ^ 1]);
      issued[s ^ 1] = true;
    }
    const bool ok_full = mbar_wait(&full[s], ph_full[s], a.spin);
    if (__syncthreads_or(!ok_full)) {
      bad = true;
      break;
    }
    ph_full[s] ^= 1;
    issued[s] = false;
    if (tid == 0) {
      tc_fence_after();
      const uint32_t As = smem_u32(Asm + s * kTcStage), Bs = smem_u32(Bsm);
#pragma unroll
      for (int m = 0; m < 6; m++) {
        const int j = m >> 1, h = m & 1;
        const uint64_t ad = sdesc(As + (j * 4 + 2 * h) * kTcChunk, kTcChunk, 128);
        const uint64_t bd = sdesc(Bs + (2 * m) * 512, 512, 128);
        tc_mma(tmem, ad, bd, kTcIdesc, m > 0 ? 1u : 0u);
      }
      tc_commit(&mma_bar);
      mma_pending = true;
    }
    const bool ok_mma = mbar_wait(&mma_bar, ph_mma, a.spin);
    if (__syncthreads_or(!ok_mma)) {
      bad = true;
      break;
    }
    ph_mma ^= 1;
    mma_pending = false;
    tc_fence_after();
    float v[32];
    tc_ld32(tmem + (uint32_t(warp * 32) << 16), v);
    const int row = tile * kTcRows + warp * 32 + lane;
    if (row < a.rows) {
      float4* o = reinterpret_cast<float4*>(a.out + size_t(row) * 32);
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
    tc_fence_before();
    __syncthreads();  // accumulator read by every warp before the next tile's MMAs
  }
  if (bad && tid == 0) {
    atomicExch(a.err, 1);
    // let copies and MMAs still in flight land before the memory is released
    for (int s = 0; s < 2; s++)
      if (issued[s]) mbar_wait(&full[s], ph_full[s], a.spin);
    if (mma_pending) mbar_wait(&mma_bar, ph_mma, a.spin);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// weight gradient: P[m, n] = sum_row X[row, m] G[row, n], m < 96, n < 32
// ---------------------------------------------------------------------------
constexpr int kWgK = 64;                                   // rows per K tile
constexpr uint32_t kWgALbo = 128 * 16;                     // A: 16 M-groups x 128 B per K chunk
constexpr uint32_t kWgBLbo = 4 * 128;                      // B: 4 N-groups x 128 B per K chunk
constexpr int kWgABytes = (kWgK / 8) * kWgALbo;            // 16 KB
constexpr int kWgBBytes = (kWgK / 8) * kWgBLbo;            // 4 KB
constexpr int kWgStage = kWgABytes + kWgBBytes;
constexpr int kWgSmem = 2 * kWgStage + 1024;

struct TcWgArgs {
  int rows;
  int rows_per_cta;  // multiple of kWgK
  const __nv_bfloat16* X0;  // [rows][32] features: h, Hd h, Ho h
  const __nv_bfloat16* X1;
  const __nv_bfloat16* X2;
  const float* G;           // [rows][32] fp32 gradient of the layer output
  float* part;              // [gridDim.x][96][32]
  int* err;
  long long spin;
};

__global__ void __launch_bounds__(128) k_tc_wgrad(TcWgArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t done[2];
  __shared__ uint32_t tslot;
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // zero both stages once: A rows 96..127 stay zero (M padding)
  for (int e = tid; e < 2 * kWgStage / 16; e += blockDim.x) reinterpret_cast<uint4*>(base)[e] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(&done[0], 1);
    mbar_init(&done[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tslot, 32);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  const __nv_bfloat16* X[3] = {a.X0, a.X1, a.X2};
  const int r_begin = blockIdx.x * a.rows_per_cta;
  const int r_end = min(a.rows, r_begin + a.rows_per_cta);
  uint32_t ph[2] = {0, 0};
  bool pending[2] = {false, false};
  bool bad = false;
  int it = 0;
  for (int r0 = r_begin; r0 < r_end; r0 += kWgK, it++) {
    const int s = it & 1;
    if (pending[s]) {  // MMAs that read this stage two tiles ago
      const bool ok = mbar_wait(&done[s], ph[s], a.spin);
      ph[s] ^= 1;
      pending[s] = false;
      if (__syncthreads_or(!ok)) {
        bad = true;
        break;
      }
    }
    uint8_t* As = base + s * kWgStage;
    uint8_t* Bs = As + kWgABytes;
    // A: unit = (feature m in 0..95, group of 8 rows); thread packs 8 rows of one feature
    for (int u = tid; u < 96 * (kWgK / 8); u += blockDim.x) {
      const int m = u % 96, g = u / 96;
      const __nv_bfloat16* src = X[m >> 5] + (m & 31);
      uint32_t w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int ra = r0 + 8 * g + 2 * q, rb = ra + 1;
        const __nv_bfloat16 va = ra < r_end ? src[size_t(ra) * 32] : __float2bfloat16_rn(0.f);
        const __nv_bfloat16 vb = rb < r_end ? src[size_t(rb) * 32] : __float2bfloat16_rn(0.f);
        w[q] = uint32_t(__bfloat16_as_ushort(va)) | (uint32_t(__bfloat16_as_ushort(vb)) << 16);
      }
      *reinterpret_cast<uint4*>(As + kmaj_off(m, 8 * g, kWgALbo, 128)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    // B: unit = (output component n in 0..31, group of 8 rows)
    for (int u = tid; u < 32 * (kWgK / 8); u += blockDim.x) {
      const int n = u % 32, g = u / 32;
      uint32_t w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int ra = r0 + 8 * g + 2 * q, rb = ra + 1;
        const float va = ra < r_end ? a.G[size_t(ra) * 32 + n] : 0.f;
        const float vb = rb < r_end ? a.G[size_t(rb) * 32 + n] : 0.f;
        w[q] = uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(va))) |
               (uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(vb))) << 16);
      }
      *reinterpret_cast<uint4*>(Bs + kmaj_off(n, 8 * g, kWgBLbo, 128)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t Aa = smem_u32(As), Ba = smem_u32(Bs);
#pragma unroll
      for (int kk = 0; kk < kWgK / 16; kk++) {
        const uint64_t ad = sdesc(Aa + (2 * kk) * kWgALbo, kWgALbo, 128);
        const uint64_t bd = sdesc(Ba + (2 * kk) * kWgBLbo, kWgBLbo, 128);
        tc_mma(tmem, ad, bd, kTcIdesc, (it > 0 || kk > 0) ? 1u : 0u);
      }
      tc_commit(&done[s]);
    }
    pending[s] = true;
  }
  // drain (also on the abort path)
  for (int s = 0; s < 2; s++)
    if (pending[s]) {
      const bool ok = mbar_wait(&done[s], ph[s], a.spin);
      if (!ok) bad = true;
    }
  if (__syncthreads_or(bad)) {
    if (tid == 0) atomicExch(a.err, 1);
  } else if (warp < 3) {
    tc_fence_after();
    float v[32];
    tc_ld32(tmem + (uint32_t(warp * 32) << 16), v);
    const int m = warp * 32 + lane;  // < 96
    float* p = a.part + (size_t(blockIdx.x) * 96 + m) * 32;
    const bool empty = r_begin >= r_end;
#pragma unroll
    for (int q = 0; q < 32; q++) p[q] = empty ? 0.f : v[q];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

// dW (complex, accumulated into G) from the real partials P (FP64 sum over CTAs).
// forward layer: dW_j[co][c] = sum G[co] conj(f_j[c]);
// adjoint layer: dW_j[c][c'] = s_j sum conj(G[c']) f_j[c],  s = (+, +, -).
__global__ void k_tc_wgrad_fin(int nparts, const float* __restrict__ part, int adj, float2* __restrict__ Gw) {
  // one warp per weight entry e = j * 256 + a * 16 + b (weight [j][a][b]); lanes stride over the partials
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (e >= 3 * 256) return;
  const int j = e >> 8, ia = (e >> 4) & 15, ib = e & 15;
  // forward: a = co (G index), b = c (feature index); adjoint: a = c (feature), b = c' (G index)
  const int fc = adj ? ia : ib, gc = adj ? ib : ia;
  const int mr = 32 * j + 2 * fc, mi = mr + 1, nr = 2 * gc, ni = nr + 1;
  double rr = 0, ii = 0, ri = 0, ir = 0;  // P[m_x][n_y] sums
  for (int k = lane; k < nparts; k += 32) {
    const float* p = part + size_t(k) * 96 * 32;
    rr += p[mr * 32 + nr];
    ii += p[mi * 32 + ni];
    ri += p[mr * 32 + ni];
    ir += p[mi * 32 + nr];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    ii += __shfl_xor_sync(0xffffffffu, ii, o);
    ri += __shfl_xor_sync(0xffffffffu, ri, o);
    ir += __shfl_xor_sync(0xffffffffu, ir, o);
  }
  if (lane) return;
  double re = rr + ii, im;
  if (!adj) {
    im = ri - ir;  // Gi fr - Gr fi
  } else {
    im = ir - ri;  // Gr fi - Gi fr
    if (j == 2) {
      re = -re;
      im = -im;
    }
  }
  Gw[e] = make_float2(Gw[e].x + float(re), Gw[e].y + float(im));
}

// ---------------------------------------------------------------------------
// hop features in bf16 rows for the GEMMs: Xh = h, Xa = Hd h, Xb = Ho h
// (16 channels, rows = (sample, site, spin), row = 32 bf16 = re, im interleaved)
// ---------------------------------------------------------------------------
__global__ void k_tc_hops_bf(int B, int Ns, int per, const int* __restrict__ nbr, const M32* __restrict__ H,
                             const float2* __restrict__ h, __nv_bfloat162* __restrict__ Xh,
                             __nv_bfloat162* __restrict__ Xa, __nv_bfloat162* __restrict__ Xb) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)B * Ns * 16) return;
  const int c = int(idx & 15);
  const long long bi = idx >> 4;
  const int i = int(bi % Ns);
  const int b = int(bi / Ns);
  const int blk = i / per;
  float2 a0 = make_float2(0.f, 0.f), a1 = a0, o0 = a0, o1 = a0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int j = __ldg(nbr + k * Ns + i);
    if (j / per != blk) continue;
    const M32 m = H[k * Ns + i];
    const float2* hj = h + (size_t(b) * Ns + j) * 32 + c;
    const float2 y0 = hj[0], y1 = hj[16];
    a0.x += m.r0.x * y0.x - m.r0.y * y0.y;  a0.y += m.r0.x * y0.y + m.r0.y * y0.x;  // h00 y0
    a1.x += m.r1.z * y1.x - m.r1.w * y1.y;  a1.y += m.r1.z * y1.y + m.r1.w * y1.x;  // h11 y1
    o0.x += m.r0.z * y1.x - m.r0.w * y1.y;  o0.y += m.r0.z * y1.y + m.r0.w * y1.x;  // h01 y1
    o1.x += m.r1.x * y0.x - m.r1.y * y0.y;  o1.y += m.r1.x * y0.y + m.r1.y * y0.x;  // h10 y0
  }
  const size_t o = size_t(bi) * 32 + c;  // spin 0 row element c; spin 1 at +16
  const float2 s0 = h[o], s1 = h[o + 16];
  Xh[o] = __floats2bfloat162_rn(s0.x, s0.y);
  Xh[o + 16] = __floats2bfloat162_rn(s1.x, s1.y);
  Xa[o] = __floats2bfloat162_rn(a0.x, a0.y);
  Xa[o + 16] = __floats2bfloat162_rn(a1.x, a1.y);
  Xb[o] = __floats2bfloat162_rn(o0.x, o0.y);
  Xb[o + 16] = __floats2bfloat162_rn(o1.x, o1.y);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// rows x 32 bf16, box of 8 elements (16 B) x 128 rows
static int make_map(CUtensorMap* m, const void* ptr, long long rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(QED3_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {32, cuuint64_t(rows)};
  const cuuint64_t strides[1] = {64};
  const cuuint32_t box[2] = {8, kTcRows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(QED3_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return QED3_OK;
}

int TcWork::ensure(long long rows_needed, int sm_count) {
  if (rows_needed <= rows && err) return QED3_OK;
  release();
  const size_t n = size_t(rows_needed) * 32;
  QED3_CUDA_TRY(cudaMalloc(&Xh, n * sizeof(__nv_bfloat16)));
  QED3_CUDA_TRY(cudaMalloc(&Xa, n * sizeof(__nv_bfloat16)));
  QED3_CUDA_TRY(cudaMalloc(&Xb, n * sizeof(__nv_bfloat16)));
  nparts = 4 * sm_count;  // 4 CTAs per SM (41 KB of shared memory each) hide the staging loads
  QED3_CUDA_TRY(cudaMalloc(&part, size_t(nparts) * 96 * 32 * sizeof(float)));
  QED3_CUDA_TRY(cudaMalloc(&err, sizeof(int)));
  QED3_CUDA_TRY(cudaMemset(err, 0, sizeof(int)));
  rows = rows_needed;
  sms = sm_count;
  return QED3_OK;
}

void TcWork::release() {
  void* p[] = {Xh, Xa, Xb, part, err};
  for (void* x : p)
    if (x) cudaFree(x);
  Xh = Xa = Xb = nullptr;
  part = nullptr;
  err = nullptr;
  rows = 0;
}

int tc_hops(TcWork& w, const qed3_dirac_s* d, const M32* H, int per, int B, const float2* h, cudaStream_t st) {
  const int Ns = d->Ns;
  const long long n = (long long)B * Ns * 16;
  k_tc_hops_bf<<<int((n + 255) / 256), 256, 0, st>>>(B, Ns, per, d->lat->dev.nbr, H, h,
                                                      reinterpret_cast<__nv_bfloat162*>(w.Xh),
                                                      reinterpret_cast<__nv_bfloat162*>(w.Xa),
                                                      reinterpret_cast<__nv_bfloat162*>(w.Xb));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int tc_mix(TcWork& w, long long rows, const float2* W, int adj, float* out, cudaStream_t st) {
  CUtensorMap m0, m1, m2;
  int rc;
  if ((rc = make_map(&m0, w.Xh, rows)) || (rc = make_map(&m1, w.Xa, rows)) || (rc = make_map(&m2, w.Xb, rows)))
    return rc;
  static bool attr = false;
  if (!attr) {
    QED3_CUDA_TRY(cudaFuncSetAttribute(k_tc_mix, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcMixSmem));
    attr = true;
  }
  TcMixArgs a{};
  a.rows = int(rows);
  a.ntiles = int((rows + kTcRows - 1) / kTcRows);
  a.W = W;
  a.adj = adj;
  a.out = out;
  a.err = w.err;
  a.spin = 2000000LL;
  const int grid = std::min(a.ntiles, 3 * w.sms);
  k_tc_mix<<<grid, 128, kTcMixSmem, st>>>(m0, m1, m2, a);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int tc_wgrad(TcWork& w, long long rows, const float* G, int adj, float2* Gw, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    QED3_CUDA_TRY(cudaFuncSetAttribute(k_tc_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmem));
    attr = true;
  }
  TcWgArgs a{};
  a.rows = int(rows);
  const long long per = (rows + w.nparts - 1) / w.nparts;
  a.rows_per_cta = int((per + kWgK - 1) / kWgK * kWgK);
  a.X0 = reinterpret_cast<const __nv_bfloat16*>(w.Xh);
  a.X1 = reinterpret_cast<const __nv_bfloat16*>(w.Xa);
  a.X2 = reinterpret_cast<const __nv_bfloat16*>(w.Xb);
  a.G = G;
  a.part = w.part;
  a.err = w.err;
  a.spin = 2000000LL;
  k_tc_wgrad<<<w.nparts, 128, kWgSmem, st>>>(a);
  k_tc_wgrad_fin<<<3 * 256 / 8, 256, 0, st>>>(w.nparts, w.part, adj, Gw);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int tc_check(TcWork& w, cudaStream_t st) {
  int e = 0;
  QED3_CUDA_TRY(cudaMemcpyAsync(&e, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  if (e) {
    QED3_CUDA_TRY(cudaMemset(w.err, 0, sizeof(int)));
    return fail(QED3_ERR_TIMEOUT, "tensor-core kernel gave up waiting on an mbarrier");
  }
  return QED3_OK;
}

}  // namespace qed3
