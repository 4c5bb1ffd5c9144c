// Learned gauge-covariant preconditioner: training (hand-written forward,
// backward and Adam kernels) and the collapsed form used by the solver.
//
// No counterpart in the reference.  Fields are complex fp32, layout
// [B][Ns][2 spins][C] in the solver's internal (space-filling-curve) order:
// a (sample, site, spin) row holds its C channels contiguously, the row of
// the channel-mixing GEMMs.
// The block mask (hops only between sites of the same `per`-sized block)
// matches the persistent solver's per-SM ownership, so the preconditioner it
// learns is applied there with block-local communication only.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <random>
#include <vector>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"
#include "lpc_impl.h"

namespace qed3 {

static inline int nblk(long long n, int t = 256) { return int((n + t - 1) / t); }

__device__ __forceinline__ float2 cmf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 caf(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cjf(float2 a) { return make_float2(a.x, -a.y); }

// ---- hop features: fa = Hd(h), fb = Ho(h) per channel, in-block neighbours only
__global__ void k_lpc_hops(int B, int Ns, int C, int per, const int* __restrict__ nbr, const M32* __restrict__ H,
                           const float2* __restrict__ h, float2* __restrict__ fa, float2* __restrict__ fb) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)B * Ns * C) return;
  const int c = int(idx % C);
  const long long bi = idx / C;
  const int i = int(bi % Ns);
  const int b = int(bi / Ns);
  const int blk = i / per;
  float2 a0 = make_float2(0.f, 0.f), a1 = a0, o0 = a0, o1 = a0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int j = __ldg(nbr + k * Ns + i);
    if (j / per != blk) continue;
    const M32 m = H[k * Ns + i];
    const float2* hj = h + (size_t(b) * Ns + j) * 2 * C + c;
    const float2 y0 = hj[0], y1 = hj[C];
    a0 = caf(a0, cmf(make_float2(m.r0.x, m.r0.y), y0));  // h00 y0
    a1 = caf(a1, cmf(make_float2(m.r1.z, m.r1.w), y1));  // h11 y1
    o0 = caf(o0, cmf(make_float2(m.r0.z, m.r0.w), y1));  // h01 y1
    o1 = caf(o1, cmf(make_float2(m.r1.x, m.r1.y), y0));  // h10 y0
  }
  const size_t o = size_t(bi) * 2 * C + c;
  fa[o] = a0;
  fa[o + C] = a1;
  fb[o] = o0;
  fb[o + C] = o1;
}

// ---- channel mixing of one layer (fp32 SIMT reference form) -------------------
// adj = 0: out[c]  = sum_c' W0[c,c'] h[c'] + W1[c,c'] fa[c'] + W2[c,c'] fb[c']   (Cin -> Cout)
// adj = 1: out[c'] = sum_c conj(W0[c,c']) h[c] + conj(W1) fa[c] - conj(W2) fb[c]  (Cout -> Cin)
__global__ void k_lpc_mix(int B, int Ns, int Cin, int Cout, int adj, const float2* __restrict__ W,
                          const float2* __restrict__ h, const float2* __restrict__ fa, const float2* __restrict__ fb,
                          float2* __restrict__ out) {
  const int Co = adj ? Cin : Cout, Ci = adj ? Cout : Cin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)B * Ns * Co) return;
  const int co = int(idx % Co);
  const long long bi = idx / Co;
  float2 s0 = make_float2(0.f, 0.f), s1 = s0;
  for (int ci = 0; ci < Ci; ci++) {
    const size_t f = size_t(bi) * 2 * Ci + ci;  // spin 0; spin 1 at f + Ci
    float2 w0, w1, w2;
    if (!adj) {
      w0 = W[(0 * Cout + co) * Cin + ci];
      w1 = W[(1 * Cout + co) * Cin + ci];
      w2 = W[(2 * Cout + co) * Cin + ci];
    } else {
      w0 = cjf(W[(0 * Cout + ci) * Cin + co]);
      w1 = cjf(W[(1 * Cout + ci) * Cin + co]);
      const float2 t = cjf(W[(2 * Cout + ci) * Cin + co]);
      w2 = make_float2(-t.x, -t.y);
    }
    s0 = caf(s0, caf(cmf(w0, h[f]), caf(cmf(w1, fa[f]), cmf(w2, fb[f]))));
    s1 = caf(s1, caf(cmf(w0, h[f + Ci]), caf(cmf(w1, fa[f + Ci]), cmf(w2, fb[f + Ci]))));
  }
  out[size_t(bi) * 2 * Co + co] = s0;
  out[size_t(bi) * 2 * Co + Co + co] = s1;
}

// ---- weight gradient of one layer: partial sums over row chunks --------------
// adj = 0: dW_j[c,c'] += sum G[c] conj(f_j[c'])       (G: Cout ch, f: Cin ch)
// adj = 1: dW_j[c,c'] += sum conj(G[c']) f'_j[c]      (G: Cin ch, f: Cout ch; f'_2 = -fb)
__global__ void k_lpc_wgrad(int rows, int Cin, int Cout, int adj, const float2* __restrict__ G,
                            const float2* __restrict__ h, const float2* __restrict__ fa, const float2* __restrict__ fb,
                            int chunk, double2* __restrict__ part) {
  const int nent = 3 * Cout * Cin;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nent) return;
  const int j = e / (Cout * Cin), c = (e / Cin) % Cout, cp = e % Cin;
  const float2* f = j == 0 ? h : (j == 1 ? fa : fb);
  const float sg = (adj && j == 2) ? -1.f : 1.f;
  const int Cg = adj ? Cin : Cout, Cf = adj ? Cout : Cin;
  const int cg = adj ? cp : c, cf = adj ? c : cp;
  const long long r0 = (long long)blockIdx.y * chunk, r1 = min((long long)rows, r0 + chunk);
  double ax = 0.0, ay = 0.0;
  for (long long r = r0; r < r1; r++) {
    for (int s = 0; s < 2; s++) {
      const float2 g = G[(size_t(r) * 2 + s) * Cg + cg];
      const float2 x = f[(size_t(r) * 2 + s) * Cf + cf];
      if (!adj) {  // g conj(x)
        ax += double(g.x) * x.x + double(g.y) * x.y;
        ay += double(g.y) * x.x - double(g.x) * x.y;
      } else {  // conj(g) x
        ax += double(g.x) * x.x + double(g.y) * x.y;
        ay += double(g.x) * x.y - double(g.y) * x.x;
      }
    }
  }
  part[size_t(blockIdx.y) * nent + e] = make_double2(sg * ax, sg * ay);
}

// Weight gradient of a layer with one 1-channel side (the 1 -> 16 layer and
// its adjoint): thread (rr, c) of a 16 x 16 block walks rows rr, rr+16, ... of
// the block's chunk for wide channel c; the 16 row lanes are summed in shared
// memory.  Entry e = 16 j + c.
// adj = 0: dW_j[c] += sum G[c] conj(f_j)      (G wide, f narrow)
// adj = 1: dW_j[c] += s_j sum conj(G) f_j[c]  (G narrow, f wide; s = +, +, -)
__global__ void __launch_bounds__(256) k_lpc_wgrad_narrow(long long rows, int adj, const float2* __restrict__ G,
                                                          const float2* __restrict__ h,
                                                          const float2* __restrict__ fa,
                                                          const float2* __restrict__ fb, int chunk,
                                                          double2* __restrict__ part) {
  __shared__ float2 sh[16][48];
  const int c = threadIdx.x & 15, rr = threadIdx.x >> 4;
  const float2* f[3] = {h, fa, fb};
  float2 acc[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  const long long r0 = (long long)blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
  for (long long r = r0 + rr; r < r1; r += 16) {
    if (!adj) {
      const float2 g = G[r * 16 + c];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const float2 x = f[j][r];  // g conj(x)
        acc[j].x += g.x * x.x + g.y * x.y;
        acc[j].y += g.y * x.x - g.x * x.y;
      }
    } else {
      const float2 g = G[r];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const float2 x = f[j][r * 16 + c];  // conj(g) x
        acc[j].x += g.x * x.x + g.y * x.y;
        acc[j].y += g.x * x.y - g.y * x.x;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 3; j++) sh[rr][16 * j + c] = acc[j];
  __syncthreads();
  if (threadIdx.x < 48) {
    const int e = threadIdx.x, j = e >> 4;
    double x = 0, y = 0;
    for (int q = 0; q < 16; q++) {
      x += sh[q][e].x;
      y += sh[q][e].y;
    }
    const double sg = (adj && j == 2) ? -1.0 : 1.0;
    part[size_t(blockIdx.x) * 48 + e] = make_double2(sg * x, sg * y);
  }
}

// G[e] += sum over chunks of the FP64 partials: one warp per entry, lanes
// stride over the chunks (fixed order, deterministic)
__global__ void k_lpc_wgrad_sum(int nent, int nchunks, const double2* __restrict__ part, float2* __restrict__ G) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (e >= nent) return;
  double x = 0, y = 0;
  for (int k = lane; k < nchunks; k += 32) {
    x += part[size_t(k) * nent + e].x;
    y += part[size_t(k) * nent + e].y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
  }
  if (lane == 0) G[e] = make_float2(G[e].x + float(x), G[e].y + float(y));
}

// z = a^2 r + g
__global__ void k_lpc_out(long long n, const float2* __restrict__ aw, const float2* __restrict__ r,
                          const float2* __restrict__ g, float2* __restrict__ z) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a2 = aw[0].x * aw[0].x;
  z[i] = make_float2(a2 * r[i].x + g[i].x, a2 * r[i].y + g[i].y);
}

// per-sample dot products for the loss: P = <z, r>, Q = Re<z, Az>, E = Re<e, r>, D = Re<G, r>
__global__ void k_lpc_dots(int n, const float2* __restrict__ z, const float2* __restrict__ r,
                           const float2* __restrict__ az, const float2* __restrict__ e, double* __restrict__ part) {
  __shared__ double sh[32 * 4];
  double v[4] = {0, 0, 0, 0};
  const size_t base = size_t(blockIdx.y) * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 zi = z[base + i], ri = r[base + i], ai = az[base + i];
    v[0] += double(zi.x) * ri.x + double(zi.y) * ri.y;  // Re conj(z) r
    v[1] += double(zi.x) * ri.y - double(zi.y) * ri.x;  // Im conj(z) r
    v[2] += double(zi.x) * ai.x + double(zi.y) * ai.y;  // Re conj(z) Az
    if (e) {
      const float2 ei = e[base + i];
      v[3] += double(ei.x) * ri.x + double(ei.y) * ri.y;
    }
  }
  block_sum<4>(v, sh);
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; q++) part[(size_t(blockIdx.y) * gridDim.x + blockIdx.x) * 4 + q] = v[q];
}

// G_z = alpha_s r + beta_s Az  (alpha complex, beta real, per sample)
__global__ void k_lpc_gz(int n, int B, const double* __restrict__ coef, const float2* __restrict__ r,
                         const float2* __restrict__ az, float2* __restrict__ gz) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * B) return;
  const int b = int(idx / n);
  const float2 al = make_float2(float(coef[3 * b]), float(coef[3 * b + 1]));
  const float be = float(coef[3 * b + 2]);
  const float2 t = cmf(al, r[idx]);
  gz[idx] = make_float2(t.x + be * az[idx].x, t.y + be * az[idx].y);
}

__global__ void k_lpc_adam(int n, float2* __restrict__ W, const float2* __restrict__ G, float2* __restrict__ m,
                           float2* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 g = G[i];
  float2 mi = m[i], vi = v[i], w = W[i];
  mi.x = b1 * mi.x + (1 - b1) * g.x;
  mi.y = b1 * mi.y + (1 - b1) * g.y;
  vi.x = b2 * vi.x + (1 - b2) * g.x * g.x;
  vi.y = b2 * vi.y + (1 - b2) * g.y * g.y;
  w.x -= lr * (mi.x / c1) / (sqrtf(vi.x / c2) + eps);
  w.y -= lr * (mi.y / c1) / (sqrtf(vi.y / c2) + eps);
  m[i] = mi;
  v[i] = vi;
  W[i] = w;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int ensure_batch(qed3_lpc_s* L, int B) {
  if (B <= L->bmax) return QED3_OK;
  for (float2* p : L->act)
    if (p) cudaFree(p);
  L->act.clear();
  float2* ptrs[] = {L->fa, L->fb, L->tmp, L->gz, L->az, L->mid, L->bR, L->bE};
  for (float2* p : ptrs)
    if (p) cudaFree(p);
  L->bR = L->bE = nullptr;
  const size_t cf = size_t(B) * L->Ns * L->C * 2;  // complex entries of a C-channel field
  const size_t c1 = size_t(B) * L->Ns * 2;
  // h_1..h_LG, g_{LG-1}..g_0, and gradients of the same
  for (int k = 0; k < 2 * L->LG; k++) {
    float2* p;
    QED3_CUDA_TRY(cudaMalloc(&p, cf * sizeof(float2)));
    L->act.push_back(p);
  }
  QED3_CUDA_TRY(cudaMalloc(&L->fa, cf * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->fb, cf * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->tmp, cf * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->mid, cf * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->gz, c1 * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->az, c1 * sizeof(float2)));
  L->bmax = B;
  return QED3_OK;
}

void lpc_destroy(qed3_lpc_s* L) {
  if (!L) return;
  for (float2* p : L->act)
    if (p) cudaFree(p);
  void* ptrs[] = {L->W, L->G, L->m, L->v, L->fa, L->fb, L->tmp, L->gz, L->az, L->mid, L->part, L->R, L->E, L->bR, L->bE};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (M32* p : L->cfg_H) cudaFree(p);
  for (M32* p : L->cfg_Hd) cudaFree(p);
  L->tc.release();
  delete L;
}

int lpc_create(qed3_dirac_s* d, int channels, int layers, int per, unsigned seed, qed3_lpc_s** out) {
  if (channels < 1 || channels > 64 || layers < 1 || layers > 3) return fail(QED3_ERR_ARG, "lpc: channels 1..64, layers 1..3");
  auto* L = new qed3_lpc_s;
  L->d = d;
  L->C = channels;
  L->LG = layers;
  L->Ns = d->Ns;
  L->per = per;
  int off = 0;
  for (int l = 0; l < layers; l++) {
    const int ci = (l == 0) ? 1 : channels, co = channels;
    L->cin.push_back(ci);
    L->cout.push_back(co);
    L->woff.push_back(off);
    off += 3 * ci * co;
  }
  L->nparam = off + 1;  // + a
  std::vector<float2> w(L->nparam);
  std::mt19937_64 g(seed);
  std::normal_distribution<double> nd;
  for (int l = 0; l < layers; l++) {
    const double sc = 0.3 / std::sqrt(double(L->cin[l]));
    for (int k = 0; k < 3 * L->cin[l] * L->cout[l]; k++)
      w[L->woff[l] + k] = make_float2(float(sc * nd(g) / std::sqrt(2.0)), float(sc * nd(g) / std::sqrt(2.0)));
  }
  w[off] = make_float2(0.3f, 0.f);
  QED3_CUDA_TRY(cudaMalloc(&L->W, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->G, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->m, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->v, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMalloc(&L->part, 131072 * sizeof(double)));
  QED3_CUDA_TRY(cudaMemcpy(L->W, w.data(), L->nparam * sizeof(float2), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemset(L->m, 0, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMemset(L->v, 0, L->nparam * sizeof(float2)));
  int dev = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  QED3_CUDA_TRY(cudaDeviceGetAttribute(&L->sms, cudaDevAttrMultiProcessorCount, dev));
  L->use_tc = (channels == 16 && layers == 2);
  *out = L;
  return QED3_OK;
}

int lpc_set_tensor_cores(qed3_lpc_s* L, int enable) {
  bool any = false;
  for (int l = 0; l < L->LG; l++) any = any || (L->cin[l] == 16 && L->cout[l] == 16);
  if (enable && !any) return fail(QED3_ERR_ARG, "tensor-core mixing needs a 16 -> 16 channel layer");
  L->use_tc = enable != 0;
  return QED3_OK;
}

static bool tc_layer(const qed3_lpc_s* L, int l) { return L->use_tc && L->cin[l] == 16 && L->cout[l] == 16; }

// one layer (or its adjoint) on an input field of c_in_field channels
static int layer_apply(qed3_lpc_s* L, const M32* H, int B, int l, int adj, const float2* in, float2* out,
                       cudaStream_t st) {
  if (tc_layer(L, l)) {
    const long long rows = (long long)B * L->Ns * 2;
    int rc = L->tc.ensure((long long)L->bmax * L->Ns * 2, L->sms);
    if (!rc) rc = tc_hops(L->tc, L->d, H, L->per, B, in, st);
    if (!rc) rc = tc_mix(L->tc, rows, L->W + L->woff[l], adj, reinterpret_cast<float*>(out), st);
    return rc;
  }
  const DeviceLattice& D = L->d->lat->dev;
  const int Cin = L->cin[l], Cout = L->cout[l];
  const int Cf = adj ? Cout : Cin;  // channels of the input field
  const int Co = adj ? Cin : Cout;
  k_lpc_hops<<<nblk((long long)B * L->Ns * Cf), 256, 0, st>>>(B, L->Ns, Cf, L->per, D.nbr, H, in, L->fa, L->fb);
  k_lpc_mix<<<nblk((long long)B * L->Ns * Co), 256, 0, st>>>(B, L->Ns, Cin, Cout, adj, L->W + L->woff[l], in, L->fa,
                                                             L->fb, out);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// weight gradient of layer l given the gradient of its output and its input
static int layer_wgrad(qed3_lpc_s* L, const M32* H, int B, int l, int adj, const float2* Gout, const float2* in,
                       cudaStream_t st) {
  if (tc_layer(L, l)) {
    const long long rows = (long long)B * L->Ns * 2;
    int rc = L->tc.ensure((long long)L->bmax * L->Ns * 2, L->sms);
    if (!rc) rc = tc_hops(L->tc, L->d, H, L->per, B, in, st);
    if (!rc) rc = tc_wgrad(L->tc, rows, reinterpret_cast<const float*>(Gout), adj, L->G + L->woff[l], st);
    return rc;
  }
  const DeviceLattice& D = L->d->lat->dev;
  const int Cin = L->cin[l], Cout = L->cout[l];
  const int Cf = adj ? Cout : Cin;
  k_lpc_hops<<<nblk((long long)B * L->Ns * Cf), 256, 0, st>>>(B, L->Ns, Cf, L->per, D.nbr, H, in, L->fa, L->fb);
  if (Cin == 1 && Cout == 16) {
    const long long rows2 = (long long)B * L->Ns * 2;  // (sample, site, spin) rows
    const int chunk = int(std::max<long long>(512, (rows2 + 1023) / 1024));
    const int nch = int((rows2 + chunk - 1) / chunk);
    k_lpc_wgrad_narrow<<<nch, 256, 0, st>>>(rows2, adj, Gout, in, L->fa, L->fb, chunk,
                                              reinterpret_cast<double2*>(L->part));
    k_lpc_wgrad_sum<<<nblk(48 * 32), 256, 0, st>>>(48, nch, reinterpret_cast<double2*>(L->part), L->G + L->woff[l]);
    QED3_CUDA_TRY(cudaGetLastError());
    return QED3_OK;
  }
  const int rows = B * L->Ns;
  const int nent = 3 * Cin * Cout;
  const int nchunks = std::max(1, std::min(65536 / (2 * nent), rows / 256 + 1));
  const int chunk = (rows + nchunks - 1) / nchunks;
  dim3 grid(nblk(nent, 128), nchunks);
  k_lpc_wgrad<<<grid, 128, 0, st>>>(rows, Cin, Cout, adj, Gout, in, L->fa, L->fb, chunk,
                                    reinterpret_cast<double2*>(L->part));
  k_lpc_wgrad_sum<<<nblk((long long)nent * 32), 256, 0, st>>>(nent, nchunks, reinterpret_cast<double2*>(L->part),
                                                              L->G + L->woff[l]);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// z = N(r) for B fields r (1 channel) with the hop blocks H of one operator
static int forward_H(qed3_lpc_s* L, const M32* H, int B, const float2* r, float2* z, cudaStream_t st) {
  int rc = ensure_batch(L, B);
  if (rc) return rc;
  const int LG = L->LG;
  // act[0..LG-1] = h_1..h_LG ; act[LG..2LG-1] = g_{LG-1}..g_0 (g_0 has 1 channel)
  const float2* in = r;
  for (int l = 0; l < LG; l++) {
    if ((rc = layer_apply(L, H, B, l, 0, in, L->act[l], st))) return rc;
    in = L->act[l];
  }
  for (int l = LG - 1; l >= 0; l--) {
    float2* out = L->act[LG + (LG - 1 - l)];
    if ((rc = layer_apply(L, H, B, l, 1, in, out, st))) return rc;
    in = out;
  }
  const long long n = (long long)B * L->Ns * 2;
  k_lpc_out<<<nblk(n), 256, 0, st>>>(n, L->W + (L->nparam - 1), r, in, z);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int lpc_forward(qed3_lpc_s* L, int B, const float2* r, float2* z, cudaStream_t st) {
  const int rc = forward_H(L, L->d->H32, B, r, z, st);
  if (rc || !L->use_tc) return rc;
  return tc_check(L->tc, st);
}

// loss and parameter gradient (accumulated into L->G after zeroing) for pairs
// (r, e) that belong to the operator whose hop blocks are H (fp32) and whose
// D, D^dag act through `d`.
static int loss_grad_H(qed3_lpc_s* L, qed3_dirac_s* d, const M32* H, const M32* Hdag, int B, const float2* r,
                       const float2* e, double* loss, cudaStream_t st) {
  int rc = ensure_batch(L, B);
  if (rc) return rc;
  const int Ns = L->Ns, LG = L->LG;
  float2* z = L->tmp;  // 1-channel use of tmp
  if ((rc = forward_H(L, H, B, r, z, st))) return rc;
  // A z = D^dag D z (fp32 field apply on [B][Ns] float4 fields)
  if ((rc = dirac_apply32_blocks(d, H, L->mid, z, B, st))) return rc;
  if ((rc = dirac_apply32_blocks(d, Hdag, L->az, L->mid, B, st))) return rc;
  const int n = Ns * 2;  // complex entries per sample
  const int gx = 64;
  k_lpc_dots<<<dim3(gx, B), 256, 0, st>>>(n, z, r, L->az, e, L->part);
  QED3_CUDA_TRY(cudaGetLastError());
  std::vector<double> h(size_t(gx) * B * 4);
  QED3_CUDA_TRY(cudaMemcpyAsync(h.data(), L->part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<double> coef(3 * size_t(B));
  double Ltot = 0;
  for (int b = 0; b < B; b++) {
    double Pr = 0, Pi = 0, Q = 0, E = 0;
    for (int k = 0; k < gx; k++) {
      const double* p = &h[(size_t(b) * gx + k) * 4];
      Pr += p[0];
      Pi += p[1];
      Q += p[2];
      E += p[3];
    }
    const double P2 = Pr * Pr + Pi * Pi;
    Ltot += 1.0 - P2 / (Q * E);
    // G_z = -2 (conj(P) r Q - |P|^2 A z) / (Q^2 E) / B
    const double s = 1.0 / (Q * Q * E * B);
    coef[3 * b] = -2.0 * Pr * Q * s;
    coef[3 * b + 1] = 2.0 * Pi * Q * s;  // conj(P) = Pr - i Pi, times -2
    coef[3 * b + 2] = 2.0 * P2 * s;
  }
  *loss = Ltot / B;
  double* dcoef = L->part + 120000;
  QED3_CUDA_TRY(cudaMemcpyAsync(dcoef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  k_lpc_gz<<<nblk((long long)n * B), 256, 0, st>>>(n, B, dcoef, r, L->az, L->gz);
  QED3_CUDA_TRY(cudaMemsetAsync(L->G, 0, L->nparam * sizeof(float2), st));
  // d/da: 2a Re<G_z, r>
  {
    k_lpc_dots<<<dim3(gx, 1), 256, 0, st>>>(n * B, L->gz, r, L->gz, nullptr, L->part);
    std::vector<double> hh(size_t(gx) * 4);
    QED3_CUDA_TRY(cudaMemcpyAsync(hh.data(), L->part, hh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    float2 aw;
    QED3_CUDA_TRY(cudaMemcpyAsync(&aw, L->W + (L->nparam - 1), sizeof(float2), cudaMemcpyDeviceToHost, st));
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
    double re = 0;
    for (int k = 0; k < gx; k++) re += hh[size_t(k) * 4];
    const float2 ga = make_float2(float(2.0 * aw.x * re), 0.f);
    QED3_CUDA_TRY(cudaMemcpyAsync(L->G + (L->nparam - 1), &ga, sizeof(float2), cudaMemcpyHostToDevice, st));
  }
  // backward through the adjoint chain: g_{l-1} = L_l^adj(g_l), last is l = 0
  // grads live in tmp/mid ping-pong over C-channel fields
  const float2* Gcur = L->gz;  // gradient of g_0 (1 channel)
  float2* gbuf[2] = {L->tmp, L->mid};
  int which = 0;
  for (int l = 0; l < LG; l++) {
    // input of L_l^adj is g_l (= act[LG + (LG-1-l) - 1] for l < LG-1 ... ) ; g_LG is h_LG
    const float2* in_adj = (l == LG - 1) ? L->act[LG - 1] : L->act[LG + (LG - 2 - l)];
    if ((rc = layer_wgrad(L, H, B, l, 1, Gcur, in_adj, st))) return rc;
    float2* Gnext = gbuf[which];
    which ^= 1;
    if ((rc = layer_apply(L, H, B, l, 0, Gcur, Gnext, st))) return rc;  // backward of adj = forward
    Gcur = Gnext;
  }
  // Gcur is the gradient of h_LG; backward through the forward chain
  for (int l = LG - 1; l >= 0; l--) {
    const float2* in_fwd = (l == 0) ? r : L->act[l - 1];
    if ((rc = layer_wgrad(L, H, B, l, 0, Gcur, in_fwd, st))) return rc;
    if (l > 0) {
      float2* Gnext = gbuf[which];
      which ^= 1;
      if ((rc = layer_apply(L, H, B, l, 1, Gcur, Gnext, st))) return rc;  // backward of fwd = adjoint
      Gcur = Gnext;
    }
  }
  return QED3_OK;
}

int lpc_loss_grad(qed3_lpc_s* L, int B, const float2* r, const float2* e, double* loss, cudaStream_t st) {
  const int rc = loss_grad_H(L, L->d, L->d->H32, L->d->Hd32, B, r, e, loss, st);
  if (rc || !L->use_tc) return rc;
  return tc_check(L->tc, st);
}

int lpc_adam(qed3_lpc_s* L, double lr, cudaStream_t st) {
  L->adam_t++;
  L->coef_valid = false;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, float(L->adam_t)), c2 = 1.f - std::pow(b2, float(L->adam_t));
  k_lpc_adam<<<nblk(L->nparam), 256, 0, st>>>(L->nparam, L->W, L->G, L->m, L->v, float(lr), b1, b2, 1e-8f, c1, c2);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// ---- collapsed form ------------------------------------------------------------
// G r = sum_w K_w O_w r over words w of length LG over {I, Hd, Ho}; with
// identities merged the distinct words are I, Hd, Ho (and HdHd, HdHo, HoHd,
// HoHo for LG = 2), word (a b) meaning O_a O_b (O_b applied first).
// N r = a^2 r + sum_{w w'} M_{w w'} O_w^dag O_w' r with M = K^dag K.
int lpc_word_coef(const qed3_lpc_s* L, LpcWordCoef* out) {
  if (L->LG > 2) return fail(QED3_ERR_ARG, "the collapsed (solver) form covers networks of 1 or 2 layers");
  std::vector<float2> w(L->nparam);
  QED3_CUDA_TRY(cudaMemcpy(w.data(), L->W, L->nparam * sizeof(float2), cudaMemcpyDeviceToHost));
  using cd = std::complex<double>;
  const int C = L->C;
  // word index: 0 = I, 1 = Hd, 2 = Ho, 3 + 2a + b for (O_{a+1} O_{b+1}) -> 3: HdHd 4: HdHo 5: HoHd 6: HoHo
  const int nw = L->LG == 1 ? 3 : 7;
  std::vector<std::vector<cd>> K(nw, std::vector<cd>(C, 0.0));
  auto W = [&](int l, int j, int co, int ci) {
    const float2 v = w[L->woff[l] + (j * L->cout[l] + co) * L->cin[l] + ci];
    return cd(v.x, v.y);
  };
  if (L->LG == 1) {
    for (int c = 0; c < C; c++)
      for (int j = 0; j < 3; j++) K[j][c] += W(0, j, c, 0);
  } else {
    // G r [c'] = sum_{j', j} sum_c W2_j'[c', c] W1_j[c] O_j' O_j r
    for (int cp = 0; cp < C; cp++)
      for (int jp = 0; jp < 3; jp++)
        for (int j = 0; j < 3; j++) {
          cd s = 0;
          for (int c = 0; c < C; c++) s += W(1, jp, cp, c) * W(0, j, c, 0);
          int word;
          if (jp == 0) word = j;            // I O_j
          else if (j == 0) word = jp;       // O_j' I
          else word = 3 + 2 * (jp - 1) + (j - 1);
          K[word][cp] += s;
        }
  }
  LpcWordCoef co{};
  co.nwords = nw;
  co.per = L->per;
  co.a2 = w[L->nparam - 1].x * w[L->nparam - 1].x;
  for (int a = 0; a < nw; a++)
    for (int b = 0; b < nw; b++) {
      cd s = 0;
      for (int c = 0; c < C; c++) s += std::conj(K[a][c]) * K[b][c];
      co.M[a][b] = make_float2(float(s.real()), float(s.imag()));
    }
  *out = co;
  return QED3_OK;
}

int lpc_word_coef_cached(qed3_lpc_s* L, LpcWordCoef* out) {
  if (!L->coef_valid) {
    const int rc = lpc_word_coef(L, &L->coef);
    if (rc) return rc;
    L->coef_valid = true;
  }
  *out = L->coef;
  return QED3_OK;
}

// host weights: nparam complex entries as interleaved (re, im) doubles
int lpc_get_weights(const qed3_lpc_s* L, double* w) {
  std::vector<float2> h(L->nparam);
  QED3_CUDA_TRY(cudaMemcpy(h.data(), L->W, L->nparam * sizeof(float2), cudaMemcpyDeviceToHost));
  for (int i = 0; i < L->nparam; i++) {
    w[2 * i] = h[i].x;
    w[2 * i + 1] = h[i].y;
  }
  return QED3_OK;
}

int lpc_set_weights(qed3_lpc_s* L, const double* w) {
  std::vector<float2> h(L->nparam);
  for (int i = 0; i < L->nparam; i++) h[i] = make_float2(float(w[2 * i]), float(w[2 * i + 1]));
  QED3_CUDA_TRY(cudaMemcpy(L->W, h.data(), L->nparam * sizeof(float2), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemset(L->m, 0, L->nparam * sizeof(float2)));
  QED3_CUDA_TRY(cudaMemset(L->v, 0, L->nparam * sizeof(float2)));
  L->adam_t = 0;
  L->coef_valid = false;
  return QED3_OK;
}

}  // namespace qed3

// ---- collapsed-form application on global fields (standalone) ----------------
namespace qed3 {

// fa = Hd(x), fb = Ho(x) for a 1-channel field (or only one of them)
__global__ void k_lpc_hop1(int B, int Ns, int per, const int* __restrict__ nbr, const M32* __restrict__ H,
                           const float2* __restrict__ x, float2* __restrict__ fa, float2* __restrict__ fb) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)B * Ns) return;
  const int i = int(idx % Ns);
  const int b = int(idx / Ns);
  const int blk = i / per;
  float2 a0 = make_float2(0.f, 0.f), a1 = a0, o0 = a0, o1 = a0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int j = __ldg(nbr + k * Ns + i);
    if (j / per != blk) continue;
    const M32 m = H[k * Ns + i];
    const float2 y0 = x[(size_t(b) * Ns + j) * 2], y1 = x[(size_t(b) * Ns + j) * 2 + 1];
    a0 = caf(a0, cmf(make_float2(m.r0.x, m.r0.y), y0));
    a1 = caf(a1, cmf(make_float2(m.r1.z, m.r1.w), y1));
    o0 = caf(o0, cmf(make_float2(m.r0.z, m.r0.w), y1));
    o1 = caf(o1, cmf(make_float2(m.r1.x, m.r1.y), y0));
  }
  if (fa) {
    fa[size_t(idx) * 2] = a0;
    fa[size_t(idx) * 2 + 1] = a1;
  }
  if (fb) {
    fb[size_t(idx) * 2] = o0;
    fb[size_t(idx) * 2 + 1] = o1;
  }
}

// out = sum_k c_k in_k over up to 8 complex fields (per-field complex scalar)
struct Lin8 {
  const float2* in[8];
  float2 c[8];
  int n;
};
__global__ void k_lpc_lin(long long n, Lin8 L, float2* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 s = make_float2(0.f, 0.f);
  for (int k = 0; k < L.n; k++) s = caf(s, cmf(L.c[k], L.in[k][i]));
  out[i] = s;
}

int lpc_apply_words(qed3_lpc_s* L, int B, const float2* r, float2* z, cudaStream_t st) {
  LpcWordCoef co;
  int rc = lpc_word_coef(L, &co);
  if (rc) return rc;
  rc = ensure_batch(L, B);
  if (rc) return rc;
  const DeviceLattice& D = L->d->lat->dev;
  const M32* H = L->d->H32;
  const int Ns = L->Ns, nw = co.nwords;
  const long long n = (long long)B * Ns * 2;
  // word fields f_0..f_{nw-1} and mixed g_0..g_{nw-1}: carve C-channel scratch
  if (L->C < nw) return fail(QED3_ERR_ARG, "word form needs at least as many channels as words (scratch)");
  float2* f[7] = {};
  float2* g[7] = {};
  for (int w = 0; w < nw; w++) {
    f[w] = L->act[0] + size_t(w) * n;  // act buffers hold C >= nw one-channel fields each
    g[w] = L->act[1] + size_t(w) * n;
  }
  const int gb = nblk((long long)B * Ns);
  f[0] = const_cast<float2*>(r);
  k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, r, f[1], f[2]);
  if (nw == 7) {
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, f[1], f[3], f[5]);  // Hd Hd r, Ho Hd r
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, f[2], f[4], f[6]);  // Hd Ho r, Ho Ho r
  }
  for (int w = 0; w < nw; w++) {
    Lin8 lin{};
    lin.n = nw;
    for (int k = 0; k < nw; k++) {
      lin.in[k] = f[k];
      lin.c[k] = co.M[w][k];
    }
    k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, lin, g[w]);
  }
  float2* ta = L->fa;
  float2* tb = L->fb;
  float2* u = L->mid;
  float2* vv = L->gz;
  if (nw == 7) {
    // u = g1 + Hd g3 - Ho g5 ; v = -g2 - Hd g4 + Ho g6
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, g[3], ta, nullptr);
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, g[5], nullptr, tb);
    Lin8 l1{};
    l1.n = 3;
    l1.in[0] = g[1]; l1.c[0] = make_float2(1, 0);
    l1.in[1] = ta;   l1.c[1] = make_float2(1, 0);
    l1.in[2] = tb;   l1.c[2] = make_float2(-1, 0);
    k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, l1, u);
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, g[4], ta, nullptr);
    k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, g[6], nullptr, tb);
    Lin8 l2{};
    l2.n = 3;
    l2.in[0] = g[2]; l2.c[0] = make_float2(-1, 0);
    l2.in[1] = ta;   l2.c[1] = make_float2(-1, 0);
    l2.in[2] = tb;   l2.c[2] = make_float2(1, 0);
    k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, l2, vv);
  } else {
    // u = g1 ; v = -g2
    Lin8 l1{};
    l1.n = 1; l1.in[0] = g[1]; l1.c[0] = make_float2(1, 0);
    k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, l1, u);
    Lin8 l2{};
    l2.n = 1; l2.in[0] = g[2]; l2.c[0] = make_float2(-1, 0);
    k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, l2, vv);
  }
  // z = a^2 r + g0 + Hd u + Ho v
  k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, u, ta, nullptr);
  k_lpc_hop1<<<gb, 256, 0, st>>>(B, Ns, co.per, D.nbr, H, vv, nullptr, tb);
  Lin8 lf{};
  lf.n = 4;
  lf.in[0] = r;    lf.c[0] = make_float2(co.a2, 0);
  lf.in[1] = g[0]; lf.c[1] = make_float2(1, 0);
  lf.in[2] = ta;   lf.c[2] = make_float2(1, 0);
  lf.in[3] = tb;   lf.c[3] = make_float2(1, 0);
  k_lpc_lin<<<nblk(n), 256, 0, st>>>(n, lf, z);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// ---- training data: residual / error pairs from the solver's own iterates -------
// For each source b: x* = full solve; for each snapshot k: x_k = the solver
// stopped after k iterations; pair (r_k = b - A x_k, e_k = x* - x_k), both
// scaled by 1/|r_k| and stored in internal order (fp32), tagged with the
// operator's hop blocks (copied, so the operator may change afterwards).
__global__ void k_lpc_pair(int Ns, const int* __restrict__ perm, const double2* __restrict__ b,
                           const double2* __restrict__ Ax, const double2* __restrict__ xs,
                           const double2* __restrict__ xk, double scale, float2* __restrict__ R,
                           float2* __restrict__ E) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int x = perm[i];
  for (int s = 0; s < 2; s++) {
    const double2 bb = b[2 * x + s], ax = Ax[2 * x + s], a = xs[2 * x + s], k = xk[2 * x + s];
    R[2 * i + s] = make_float2(float((bb.x - ax.x) * scale), float((bb.y - ax.y) * scale));
    E[2 * i + s] = make_float2(float((a.x - k.x) * scale), float((a.y - k.y) * scale));
  }
}

}  // namespace qed3

namespace qed3 {

__global__ void k_gauss_spinor(long long n, unsigned long long seed, double* v) {
  // Box-Muller on a counter hash: synthetic Gaussian sources for training
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long h = (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ULL ^ (seed * 0xBF58476D1CE4E5B9ULL);
  h ^= h >> 31;
  h *= 0x94D049BB133111EBULL;
  h ^= h >> 29;
  const double u1 = (double((h >> 11) & ((1ULL << 53) - 1)) + 0.5) / double(1ULL << 53);
  unsigned long long g = h * 0xD6E8FEB86659FD93ULL;
  g ^= g >> 32;
  const double u2 = double((g >> 11) & ((1ULL << 53) - 1)) / double(1ULL << 53);
  v[i] = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

__global__ void k_gather_pairs(int B, int Ns, const int* __restrict__ idx, const float2* __restrict__ R,
                               const float2* __restrict__ E, float2* __restrict__ bR, float2* __restrict__ bE) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = (long long)Ns * 2;
  if (t >= per * B) return;
  const int b = int(t / per);
  const long long o = t % per;
  bR[t] = R[size_t(idx[b]) * per + o];
  bE[t] = E[size_t(idx[b]) * per + o];
}

int lpc_collect(qed3_lpc_s* L, qed3_dirac_s* d, int nsrc, unsigned seed, const int* snaps, int nsnap, int prec) {
  if (d->Ns != L->Ns) return fail(QED3_ERR_ARG, "operator lattice differs from the preconditioner's");
  const int Ns = L->Ns;
  const size_t nd = size_t(4) * Ns;  // doubles per vector
  const int need = L->npairs + nsrc * nsnap;
  if (need > L->cap_pairs) {
    const int cap = std::max(need, 2 * L->cap_pairs);
    float2 *R2, *E2;
    QED3_CUDA_TRY(cudaMalloc(&R2, size_t(cap) * Ns * 2 * sizeof(float2)));
    QED3_CUDA_TRY(cudaMalloc(&E2, size_t(cap) * Ns * 2 * sizeof(float2)));
    if (L->npairs) {
      QED3_CUDA_TRY(cudaMemcpy(R2, L->R, size_t(L->npairs) * Ns * 2 * sizeof(float2), cudaMemcpyDeviceToDevice));
      QED3_CUDA_TRY(cudaMemcpy(E2, L->E, size_t(L->npairs) * Ns * 2 * sizeof(float2), cudaMemcpyDeviceToDevice));
    }
    if (L->R) cudaFree(L->R);
    if (L->E) cudaFree(L->E);
    L->R = R2;
    L->E = E2;
    L->cap_pairs = cap;
  }
  M32* Hc;
  QED3_CUDA_TRY(cudaMalloc(&Hc, size_t(3) * Ns * sizeof(M32)));
  QED3_CUDA_TRY(cudaMemcpy(Hc, d->H32, size_t(3) * Ns * sizeof(M32), cudaMemcpyDeviceToDevice));
  L->cfg_H.push_back(Hc);
  QED3_CUDA_TRY(cudaMalloc(&Hc, size_t(3) * Ns * sizeof(M32)));
  QED3_CUDA_TRY(cudaMemcpy(Hc, d->Hd32, size_t(3) * Ns * sizeof(M32), cudaMemcpyDeviceToDevice));
  L->cfg_Hd.push_back(Hc);
  const int cfg = int(L->cfg_H.size()) - 1;
  double *b, *xs, *xk, *ax;
  QED3_CUDA_TRY(cudaMalloc(&b, nd * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&xs, nd * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&xk, nd * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&ax, nd * sizeof(double)));
  int rc = QED3_OK;
  for (int s = 0; s < nsrc && rc == QED3_OK; s++) {
    k_gauss_spinor<<<nblk((long long)nd), 256>>>((long long)nd, 1000003ULL * seed + s, b);
    qed3_solve_params full{1e-10, 0, prec, 0.1, 0.0, 0};
    if ((rc = cg_solve(d, xs, b, &full, nullptr, 0))) break;
    for (int k = 0; k < nsnap; k++) {
      if (snaps[k] <= 0) {
        QED3_CUDA_TRY(cudaMemset(xk, 0, nd * sizeof(double)));
      } else {
        qed3_solve_params tr{1e-14, snaps[k], prec, 0.1, 0.0, 0};
        rc = cg_solve(d, xk, b, &tr, nullptr, 0);
        if (rc && rc != QED3_ERR_NOCONV) break;
        rc = QED3_OK;
      }
      if ((rc = dirac_apply_ref(d, QED3_OP_DDAGD, ax, xk, 0))) break;
      // |r_k| on the host for the normalisation
      std::vector<double> hb(nd), ha(nd);
      QED3_CUDA_TRY(cudaMemcpy(hb.data(), b, nd * sizeof(double), cudaMemcpyDeviceToHost));
      QED3_CUDA_TRY(cudaMemcpy(ha.data(), ax, nd * sizeof(double), cudaMemcpyDeviceToHost));
      double nr = 0;
      for (size_t q = 0; q < nd; q++) nr += (hb[q] - ha[q]) * (hb[q] - ha[q]);
      const int pi = L->npairs++;
      k_lpc_pair<<<nblk(Ns), 256>>>(Ns, d->lat->dev.perm, reinterpret_cast<const double2*>(b),
                                    reinterpret_cast<const double2*>(ax), reinterpret_cast<const double2*>(xs),
                                    reinterpret_cast<const double2*>(xk), 1.0 / std::sqrt(nr),
                                    L->R + size_t(pi) * Ns * 2, L->E + size_t(pi) * Ns * 2);
      L->pair_cfg.push_back(cfg);
    }
  }
  cudaFree(b);
  cudaFree(xs);
  cudaFree(xk);
  cudaFree(ax);
  QED3_CUDA_TRY(cudaDeviceSynchronize());
  return rc;
}

// Adam on the cos^2 loss; each step draws one operator, then `batch` of its
// pairs.  history[k] = loss of step k (may be NULL).
int lpc_train(qed3_lpc_s* L, int steps, int batch, double lr, unsigned seed, double* history) {
  if (L->npairs < 1) return fail(QED3_ERR_STATE, "no training pairs (call qed3_lpc_collect)");
  int rc = ensure_batch(L, batch);
  if (rc) return rc;
  const int Ns = L->Ns;
  if (!L->bR) {
    QED3_CUDA_TRY(cudaMalloc(&L->bR, size_t(L->bmax) * Ns * 2 * sizeof(float2)));
    QED3_CUDA_TRY(cudaMalloc(&L->bE, size_t(L->bmax) * Ns * 2 * sizeof(float2)));
  }
  std::vector<std::vector<int>> by_cfg(L->cfg_H.size());
  for (int p = 0; p < L->npairs; p++) by_cfg[L->pair_cfg[p]].push_back(p);
  std::vector<int> cfgs;
  for (size_t c = 0; c < by_cfg.size(); c++)
    if (!by_cfg[c].empty()) cfgs.push_back(int(c));
  std::mt19937_64 g(seed);
  int* didx;
  QED3_CUDA_TRY(cudaMalloc(&didx, batch * sizeof(int)));
  for (int it = 0; it < steps; it++) {
    const int c = cfgs[g() % cfgs.size()];
    std::vector<int> idx(batch);
    for (int b = 0; b < batch; b++) idx[b] = by_cfg[c][g() % by_cfg[c].size()];
    QED3_CUDA_TRY(cudaMemcpy(didx, idx.data(), batch * sizeof(int), cudaMemcpyHostToDevice));
    k_gather_pairs<<<nblk((long long)batch * Ns * 2), 256>>>(batch, Ns, didx, L->R, L->E, L->bR, L->bE);
    // hop features and D^dag D both use the pairs' own operator
    double loss = 0;
    rc = loss_grad_H(L, L->d, L->cfg_H[c], L->cfg_Hd[c], batch, L->bR, L->bE, &loss, 0);
    if (rc) break;
    if ((rc = lpc_adam(L, lr, 0))) break;
    if (history) history[it] = loss;
  }
  cudaFree(didx);
  if (!rc && L->use_tc) rc = tc_check(L->tc, 0);
  return rc;
}

}  // namespace qed3
