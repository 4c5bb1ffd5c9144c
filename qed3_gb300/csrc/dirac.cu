// Wilson-Dirac operator on the dual lattice: coefficient build and the
// gather-stencil apply kernels (sm_103a).
//
// Replaces the reference's host COO assembly + CSR SpMV
// (src/both_3d/dirac_ext.h:122-213, src/both_3d/sparse_dirac.h:132-151,
// src/dual/gpu_header.h:102-117).  The sparsity is fixed -- three 2x2 hop
// blocks plus a real scalar diagonal per site -- so instead of CSR
// (12 nnz/row, 20 B/nnz + gathers) each site reads its three neighbour ids,
// three 2x2 blocks and its neighbours' two-spinors: 276 B/site in FP64,
// 144 B in FP32, 128 B with bf16 spinors.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"

namespace qed3 {

using cd = std::complex<double>;

// ---------------------------------------------------------------------------
// U(1) phases: H_xy = e^{i A_xy} G_xy,  (H_yx)^dagger = e^{i A_xy} (G_yx)^dagger
// ---------------------------------------------------------------------------
__global__ void k_set_links(int Ns, const int32_t* __restrict__ hop_link, const int8_t* __restrict__ hop_sign,
                            const double* __restrict__ A, const M64* __restrict__ G, const M64* __restrict__ Gd,
                            M64* __restrict__ H, M64* __restrict__ Hd, M32* __restrict__ H32, M32* __restrict__ Hd32) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 3 * Ns) return;
  const double a = double(hop_sign[idx]) * A[hop_link[idx]];
  double s, c;
  sincos(a, &s, &c);
  const double2 ph = make_double2(c, s);
  const M64 g = G[idx], gd = Gd[idx];
  M64 h{cmul(ph, g.h00), cmul(ph, g.h01), cmul(ph, g.h10), cmul(ph, g.h11)};
  M64 hd{cmul(ph, gd.h00), cmul(ph, gd.h01), cmul(ph, gd.h10), cmul(ph, gd.h11)};
  H[idx] = h;
  Hd[idx] = hd;
  H32[idx] = M32{make_float4(float(h.h00.x), float(h.h00.y), float(h.h01.x), float(h.h01.y)),
                 make_float4(float(h.h10.x), float(h.h10.y), float(h.h11.x), float(h.h11.y))};
  Hd32[idx] = M32{make_float4(float(hd.h00.x), float(hd.h00.y), float(hd.h01.x), float(hd.h01.y)),
                  make_float4(float(hd.h10.x), float(hd.h10.y), float(hd.h11.x), float(hd.h11.y))};
}

__global__ void k_to32(int n, const M64* __restrict__ H, const M64* __restrict__ Hd, M32* __restrict__ H32,
                       M32* __restrict__ Hd32) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const M64 h = H[idx], hd = Hd[idx];
  H32[idx] = M32{make_float4(float(h.h00.x), float(h.h00.y), float(h.h01.x), float(h.h01.y)),
                 make_float4(float(h.h10.x), float(h.h10.y), float(h.h11.x), float(h.h11.y))};
  Hd32[idx] = M32{make_float4(float(hd.h00.x), float(hd.h00.y), float(hd.h01.x), float(hd.h01.y)),
                  make_float4(float(hd.h10.x), float(hd.h10.y), float(hd.h11.x), float(hd.h11.y))};
}

// ---------------------------------------------------------------------------
// Apply kernels
// ---------------------------------------------------------------------------
// Internal-order FP64: out = D in (H) or D^dagger in (Hd); nrhs fields back to back.
__global__ void __launch_bounds__(256) k_apply64(int Ns, int nrhs, const int* __restrict__ nbr,
                                                 const M64* __restrict__ H, const double* __restrict__ diag,
                                                 const S64* __restrict__ in, S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  for (int r = 0; r < nrhs; r++) {
    const Sp64 o = hop64(i, Ns, nbr, H, diag, in + size_t(r) * Ns);
    st64(out + size_t(r) * Ns, i, o);
  }
}

template <int P>
__global__ void __launch_bounds__(256) k_apply32(int Ns, int nrhs, const int* __restrict__ nbr,
                                                 const M32* __restrict__ H, const float* __restrict__ diag,
                                                 const typename LoField<P>::T* __restrict__ in,
                                                 typename LoField<P>::T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  for (int r = 0; r < nrhs; r++) {
    const Sp32 o = hop32<P>(i, Ns, nbr, H, diag, in + size_t(r) * Ns);
    LoField<P>::st(out + size_t(r) * Ns, i, o);
  }
}

// Reference-order FP64 apply: thread i handles internal site i, reads the
// reference-ordered input through perm/nbr_ref and writes out[perm[i]].
// mode 0: in ref -> out ref; 1: in ref -> out internal; 2: in internal -> out ref
__global__ void __launch_bounds__(256) k_apply64_ref(int Ns, int mode, const int* __restrict__ nbr,
                                                     const int* __restrict__ nbr_ref, const int* __restrict__ perm,
                                                     const M64* __restrict__ H, const double* __restrict__ diag,
                                                     const S64* __restrict__ in, S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int* nb = (mode == 2) ? nbr : nbr_ref;
  const int self_in = (mode == 2) ? i : __ldg(perm + i);
  const int j0 = __ldg(nb + i), j1 = __ldg(nb + Ns + i), j2 = __ldg(nb + 2 * Ns + i);
  const Sp64 a = ld64(in, self_in), b[3] = {ld64(in, j0), ld64(in, j1), ld64(in, j2)};
  const double d = __ldg(diag + i);
  Sp64 o{cscale(d, a.s0), cscale(d, a.s1)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const M64 m = H[k * Ns + i];
    o.s0 = cfma(m.h00, b[k].s0, o.s0);
    o.s0 = cfma(m.h01, b[k].s1, o.s0);
    o.s1 = cfma(m.h10, b[k].s0, o.s1);
    o.s1 = cfma(m.h11, b[k].s1, o.s1);
  }
  st64(out, (mode == 1) ? i : __ldg(perm + i), o);
}

// Field import/export between reference-order complex128 and internal fields.
template <int P>
__global__ void k_import(int Ns, int nrhs, const int* __restrict__ perm, const S64* __restrict__ in, void* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int x = perm[i];
  for (int r = 0; r < nrhs; r++) {
    const Sp64 v = ld64(in + size_t(r) * Ns, x);
    if (P == P64) {
      st64(reinterpret_cast<S64*>(out) + size_t(r) * Ns, i, v);
    } else {
      const Sp32 w{make_float2(float(v.s0.x), float(v.s0.y)), make_float2(float(v.s1.x), float(v.s1.y))};
      if (P == P32) st32(reinterpret_cast<float4*>(out) + size_t(r) * Ns, i, w);
      else stbf(reinterpret_cast<uint2*>(out) + size_t(r) * Ns, i, w);
    }
  }
}

template <int P>
__global__ void k_export(int Ns, int nrhs, const int* __restrict__ perm, const void* in, S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const int x = perm[i];
  for (int r = 0; r < nrhs; r++) {
    Sp64 v;
    if (P == P64) {
      v = ld64(reinterpret_cast<const S64*>(in) + size_t(r) * Ns, i);
    } else {
      const Sp32 w = (P == P32) ? ld32(reinterpret_cast<const float4*>(in) + size_t(r) * Ns, i)
                                : ldbf(reinterpret_cast<const uint2*>(in) + size_t(r) * Ns, i);
      v = Sp64{make_double2(w.s0.x, w.s0.y), make_double2(w.s1.x, w.s1.y)};
    }
    st64(out + size_t(r) * Ns, x, v);
  }
}

static inline int nblk(long long n, int t = 256) { return int((n + t - 1) / t); }

// Unit-norm import for the solvers: block partials of |b|^2, then every block
// of the import sums the partials in the same fixed order (one warp), divides
// b by |b| and block 0 stores |b|.  The solvers iterate on b / |b| so their
// FP32/BF16 vectors stay near unit scale whatever the scale of b (a residual
// of a right-hand side with |b_i| ~ 1e-20 would underflow in FP32, one with
// |b_i| ~ 1e20 would overflow); the export multiplies the solution by |b|.
constexpr int kNormParts = 64;  // partials read by every import block: keep them few

__global__ void k_norm_part(long long n, const double* __restrict__ in, double* __restrict__ part) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v[0] += in[i] * in[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_import_unit(int Ns, const int* __restrict__ perm, const S64* __restrict__ in,
                              const double* __restrict__ part, int nparts, S64* __restrict__ out,
                              double* __restrict__ nrm_out) {
  __shared__ double inv_s;
  if (threadIdx.x < 32) {
    double s = 0.0;
    for (int k = threadIdx.x; k < nparts; k += 32) s += part[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) {
      const double nr = sqrt(s);
      inv_s = nr > 0.0 ? 1.0 / nr : 0.0;
      if (blockIdx.x == 0) *nrm_out = nr;
    }
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const double inv = inv_s;
  Sp64 v = ld64(in, perm[i]);
  v.s0 = cscale(inv, v.s0);
  v.s1 = cscale(inv, v.s1);
  st64(out, i, v);
}

__global__ void k_export_scaled(int Ns, const int* __restrict__ perm, const S64* __restrict__ in,
                                const double* __restrict__ nrm, S64* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ns) return;
  const double s = *nrm;
  Sp64 v = ld64(in, i);
  v.s0 = cscale(s, v.s0);
  v.s1 = cscale(s, v.s1);
  st64(out, perm[i], v);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static void geom_block(const HostLattice& L, const std::vector<double>& kappa, double r, int x, int k, cd G[4]) {
  const int l = L.hop_link[3 * x + k];
  const double om = L.hop_sign[3 * x + k] * L.omega[l];
  const double al = L.alpha[3 * x + k];
  const double hk = 0.5 * kappa[l];
  const cd em(std::cos(0.5 * om), -std::sin(0.5 * om)), ep(std::cos(0.5 * om), std::sin(0.5 * om));
  const cd ua(std::cos(al), std::sin(al));
  // (kappa/2) (-r + gamma(alpha)) Omega(omega), gamma = [[0, e^{-ia}], [e^{ia}, 0]],
  // Omega = diag(e^{-i om/2}, e^{+i om/2})
  G[0] = hk * (-r) * em;
  G[1] = hk * std::conj(ua) * ep;
  G[2] = hk * ua * em;
  G[3] = hk * (-r) * ep;
}

int dirac_init_device(qed3_dirac_s* d) {
  const HostLattice& L = d->lat->host;
  const int Ns = L.n_sites, Nl = L.n_links;
  d->Ns = Ns;
  d->kappa.resize(Nl);
  // kappa_l = 2 V_l / ell_l / mean_ell, src/both_3d/dirac_dual.h:208-214
  for (int l = 0; l < Nl; l++) d->kappa[l] = 2.0 * L.link_volume[l] / L.ell[l] / L.mean_ell;
  std::vector<M64> G(size_t(3) * Ns), Gd(size_t(3) * Ns);
  std::vector<double> diag(Ns);
  std::vector<float> diag32(Ns);
  for (int i = 0; i < Ns; i++) {
    const int x = L.perm[i];
    double coeff = 0.0;
    for (int k = 0; k < 3; k++) {
      cd g[4], gy[4];
      geom_block(L, d->kappa, d->r, x, k, g);
      const int y = L.nns[3 * x + k], kb = L.hop_back[3 * x + k];
      geom_block(L, d->kappa, d->r, y, kb, gy);
      M64& m = G[size_t(k) * Ns + i];
      m.h00 = make_double2(g[0].real(), g[0].imag());
      m.h01 = make_double2(g[1].real(), g[1].imag());
      m.h10 = make_double2(g[2].real(), g[2].imag());
      m.h11 = make_double2(g[3].real(), g[3].imag());
      M64& md = Gd[size_t(k) * Ns + i];  // conjugate transpose of G_yx
      md.h00 = make_double2(gy[0].real(), -gy[0].imag());
      md.h01 = make_double2(gy[2].real(), -gy[2].imag());
      md.h10 = make_double2(gy[1].real(), -gy[1].imag());
      md.h11 = make_double2(gy[3].real(), -gy[3].imag());
      coeff += 0.5 * d->r * d->kappa[L.hop_link[3 * x + k]];
    }
    coeff += d->M5;  // src/both_3d/dirac_ext.h:193-212 (kappa_t = 0 at Nt = 1)
    diag[i] = coeff;
    diag32[i] = float(coeff);
  }
  const size_t nm = size_t(3) * Ns;
  QED3_CUDA_TRY(cudaMalloc(&d->G, nm * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&d->Gd, nm * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&d->H, nm * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&d->Hd, nm * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&d->H32, nm * sizeof(M32)));
  QED3_CUDA_TRY(cudaMalloc(&d->Hd32, nm * sizeof(M32)));
  QED3_CUDA_TRY(cudaMalloc(&d->diag, size_t(Ns) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&d->diag32, size_t(Ns) * sizeof(float)));
  QED3_CUDA_TRY(cudaMalloc(&d->A_dev, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&d->tmp_in, size_t(Ns) * sizeof(S64)));
  QED3_CUDA_TRY(cudaMalloc(&d->tmp_out, size_t(Ns) * sizeof(S64)));
  QED3_CUDA_TRY(cudaMalloc(&d->tmp_mid, size_t(Ns) * sizeof(S64)));
  QED3_CUDA_TRY(cudaMemcpy(d->G, G.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->Gd, Gd.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag, diag.data(), size_t(Ns) * sizeof(double), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag32, diag32.data(), size_t(Ns) * sizeof(float), cudaMemcpyHostToDevice));
  return QED3_OK;
}

// ---------------------------------------------------------------------------
// Dirac1fonS2 (src/dual/dirac.h:145-220) on the same 3-hop layout.  Per site x
// and hop k to y = nns[x][k]:
//   D[x,y] = -(vol_x / vbar) (r u_{x,k} - v_{x,k} . (sigma1, sigma2)) Omega(x,y) e^{iU(x,y)},
//   D[x,x] = sum_k (vol_x / vbar) (r u_{x,k} + m/3) + M5,
// vol_x the spherical area of x's triangle, vbar their mean.  u and v are the
// tables integrator/test_sorting.cc:499-594 writes (us_*, vs_*), computed here
// from the hop vectors ell_k = |x y_k| (cos alpha_k, sin alpha_k):
//   v: sum_k ell_k v_k^T = (a/sqrt 3) 1 with v_3 = -v_1 - v_2, a = sqrt(4 vbar / sqrt 3);
//   u: u_1 ell_1 + u_2 ell_2 + u_3 ell_3 = 0 with u_1 = 1, then u *= 3 / mean(u).
// ---------------------------------------------------------------------------
static double acos_clamped(double c) { return c < -1.0 ? M_PI : (c > 1.0 ? 0.0 : std::acos(c)); }

static void tables_1f(const HostLattice& L, int x, double alat, double u[3], double v[3][2]) {
  double el[3][2];
  for (int k = 0; k < 3; k++) {
    const int y = L.nns[3 * x + k];
    const double* a = &L.sites[3 * size_t(x)];
    const double* b = &L.sites[3 * size_t(y)];
    const double len = acos_clamped(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    const double al = L.alpha[3 * x + k];
    el[k][0] = len * std::cos(al);
    el[k][1] = len * std::sin(al);
  }
  // [d13 d23] (v1_c, v2_c)^T = (a/sqrt3) e_c for c = x, y
  const double d13[2] = {el[0][0] - el[2][0], el[0][1] - el[2][1]};
  const double d23[2] = {el[1][0] - el[2][0], el[1][1] - el[2][1]};
  const double det = d13[0] * d23[1] - d23[0] * d13[1];
  const double c = alat / std::sqrt(3.0);
  // inverse of [[d13x, d23x], [d13y, d23y]] = [[d23y, -d23x], [-d13y, d13x]] / det
  v[0][0] = d23[1] * c / det;
  v[1][0] = -d13[1] * c / det;
  v[0][1] = -d23[0] * c / det;
  v[1][1] = d13[0] * c / det;
  v[2][0] = -v[0][0] - v[1][0];
  v[2][1] = -v[0][1] - v[1][1];
  // [ell2 ell3] (p, q)^T = -ell1
  const double det2 = el[1][0] * el[2][1] - el[2][0] * el[1][1];
  const double p = (-el[0][0] * el[2][1] + el[2][0] * el[0][1]) / det2;
  const double q = (-el[1][0] * el[0][1] + el[0][0] * el[1][1]) / det2;
  u[0] = 1.0;
  u[1] = p;
  u[2] = q;
  const double mean = (u[0] + u[1] + u[2]) / 3.0;
  for (int k = 0; k < 3; k++) u[k] *= 3.0 / mean;
}

static void block_1f(const HostLattice& L, double r, double vbar, double alat, int x, int k, cd G[4]) {
  double u[3], v[3][2];
  tables_1f(L, x, alat, u, v);
  const double w = L.tri_area[x] / vbar;
  const double om = L.hop_sign[3 * x + k] * L.omega[L.hop_link[3 * x + k]];
  const cd em(std::cos(0.5 * om), -std::sin(0.5 * om)), ep(std::cos(0.5 * om), std::sin(0.5 * om));
  const cd gm(v[k][0], -v[k][1]), gp(v[k][0], v[k][1]);  // gamma = [[0, v0 - i v1], [v0 + i v1, 0]]
  G[0] = -w * (r * u[k]) * em;
  G[1] = w * gm * ep;
  G[2] = w * gp * em;
  G[3] = -w * (r * u[k]) * ep;
}

int dirac_use_1f(qed3_dirac_s* d, double m) {
  const HostLattice& L = d->lat->host;
  const int Ns = L.n_sites;
  double vbar = 0.0;
  for (double a : L.tri_area) vbar += a;
  vbar /= Ns;
  const double alat = std::sqrt(4.0 / std::sqrt(3.0) * vbar);
  std::vector<M64> G(size_t(3) * Ns), Gd(size_t(3) * Ns);
  std::vector<double> diag(Ns);
  std::vector<float> diag32(Ns);
  auto put = [](M64& o, const cd g[4], bool adj) {
    if (!adj) {
      o = M64{make_double2(g[0].real(), g[0].imag()), make_double2(g[1].real(), g[1].imag()),
              make_double2(g[2].real(), g[2].imag()), make_double2(g[3].real(), g[3].imag())};
    } else {  // conjugate transpose
      o = M64{make_double2(g[0].real(), -g[0].imag()), make_double2(g[2].real(), -g[2].imag()),
              make_double2(g[1].real(), -g[1].imag()), make_double2(g[3].real(), -g[3].imag())};
    }
  };
  for (int i = 0; i < Ns; i++) {
    const int x = L.perm[i];
    double u[3], v[3][2];
    tables_1f(L, x, alat, u, v);
    const double w = L.tri_area[x] / vbar;
    double dg = 0.0;
    for (int k = 0; k < 3; k++) {
      dg += w * (d->r * u[k] + m / 3.0);
      cd g[4], gy[4];
      block_1f(L, d->r, vbar, alat, x, k, g);
      block_1f(L, d->r, vbar, alat, L.nns[3 * x + k], L.hop_back[3 * x + k], gy);
      put(G[size_t(k) * Ns + i], g, false);
      put(Gd[size_t(k) * Ns + i], gy, true);
    }
    diag[i] = dg + d->M5;
    diag32[i] = float(diag[i]);
  }
  const size_t nm = size_t(3) * Ns;
  QED3_CUDA_TRY(cudaMemcpy(d->G, G.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->Gd, Gd.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag, diag.data(), size_t(Ns) * sizeof(double), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag32, diag32.data(), size_t(Ns) * sizeof(float), cudaMemcpyHostToDevice));
  d->coeffs_set = false;  // the hop blocks take the link phases at the next set_links
  return QED3_OK;
}

int dirac_free_device(qed3_dirac_s* d) {
  void* ptrs[] = {d->G, d->Gd, d->H, d->Hd, d->H32, d->Hd32, d->diag, d->diag32, d->A_dev, d->tmp_in, d->tmp_out, d->tmp_mid};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  return QED3_OK;
}

int dirac_set_links(qed3_dirac_s* d, const double* A, int on_device, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  const double* Ad = A;
  if (!on_device) {
    QED3_CUDA_TRY(cudaMemcpyAsync(d->A_dev, A, size_t(D.Nl) * sizeof(double), cudaMemcpyHostToDevice, st));
    Ad = d->A_dev;
  }
  k_set_links<<<nblk(3LL * d->Ns), 256, 0, st>>>(d->Ns, D.hop_link, D.hop_sign, Ad, d->G, d->Gd, d->H, d->Hd, d->H32,
                                                 d->Hd32);
  QED3_CUDA_TRY(cudaGetLastError());
  d->coeffs_set = true;
  return QED3_OK;
}

int dirac_set_coefficients(qed3_dirac_s* d, const double* hop, const double* diag_ref) {
  const HostLattice& L = d->lat->host;
  const int Ns = d->Ns;
  std::vector<M64> H(size_t(3) * Ns), Hd(size_t(3) * Ns);
  std::vector<double> diag(Ns);
  std::vector<float> diag32(Ns);
  auto blk = [&](int x, int k, int e) { return cd(hop[(size_t(x) * 3 + k) * 8 + 2 * e], hop[(size_t(x) * 3 + k) * 8 + 2 * e + 1]); };
  for (int i = 0; i < Ns; i++) {
    const int x = L.perm[i];
    diag[i] = diag_ref[x];
    diag32[i] = float(diag_ref[x]);
    for (int k = 0; k < 3; k++) {
      const int y = L.nns[3 * x + k], kb = L.hop_back[3 * x + k];
      M64& m = H[size_t(k) * Ns + i];
      m.h00 = make_double2(blk(x, k, 0).real(), blk(x, k, 0).imag());
      m.h01 = make_double2(blk(x, k, 1).real(), blk(x, k, 1).imag());
      m.h10 = make_double2(blk(x, k, 2).real(), blk(x, k, 2).imag());
      m.h11 = make_double2(blk(x, k, 3).real(), blk(x, k, 3).imag());
      M64& md = Hd[size_t(k) * Ns + i];
      md.h00 = make_double2(blk(y, kb, 0).real(), -blk(y, kb, 0).imag());
      md.h01 = make_double2(blk(y, kb, 2).real(), -blk(y, kb, 2).imag());
      md.h10 = make_double2(blk(y, kb, 1).real(), -blk(y, kb, 1).imag());
      md.h11 = make_double2(blk(y, kb, 3).real(), -blk(y, kb, 3).imag());
    }
  }
  const size_t nm = size_t(3) * Ns;
  QED3_CUDA_TRY(cudaMemcpy(d->H, H.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->Hd, Hd.data(), nm * sizeof(M64), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag, diag.data(), size_t(Ns) * sizeof(double), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(d->diag32, diag32.data(), size_t(Ns) * sizeof(float), cudaMemcpyHostToDevice));
  k_to32<<<nblk(nm), 256>>>(int(nm), d->H, d->Hd, d->H32, d->Hd32);
  QED3_CUDA_TRY(cudaGetLastError());
  QED3_CUDA_TRY(cudaDeviceSynchronize());
  d->coeffs_set = true;
  return QED3_OK;
}

int dirac_apply_ref(qed3_dirac_s* d, int op, double* out, const double* in, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  const int Ns = d->Ns;
  const S64* vin = reinterpret_cast<const S64*>(in);
  S64* vout = reinterpret_cast<S64*>(out);
  const int g = nblk(Ns);
  if (op == QED3_OP_D || op == QED3_OP_DDAG) {
    if (in == out) {  // the stencil gathers: never in place
      QED3_CUDA_TRY(cudaMemcpyAsync(d->tmp_in, in, size_t(Ns) * sizeof(S64), cudaMemcpyDeviceToDevice, st));
      vin = d->tmp_in;
    }
    k_apply64_ref<<<g, 256, 0, st>>>(Ns, 0, D.nbr, D.nbr_ref, D.perm, op == QED3_OP_D ? d->H : d->Hd, d->diag, vin,
                                     vout);
  } else {
    const M64* first = (op == QED3_OP_DDAGD) ? d->H : d->Hd;
    const M64* second = (op == QED3_OP_DDAGD) ? d->Hd : d->H;
    k_apply64_ref<<<g, 256, 0, st>>>(Ns, 1, D.nbr, D.nbr_ref, D.perm, first, d->diag, vin, d->tmp_mid);
    k_apply64_ref<<<g, 256, 0, st>>>(Ns, 2, D.nbr, D.nbr_ref, D.perm, second, d->diag, d->tmp_mid, vout);
  }
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int field_import(qed3_dirac_s* d, int prec, void* field, const double* in_ref, int nrhs, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  const int g = nblk(d->Ns);
  const S64* in = reinterpret_cast<const S64*>(in_ref);
  if (prec == QED3_PREC_F64) k_import<P64><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, in, field);
  else if (prec == QED3_PREC_F32) k_import<P32><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, in, field);
  else k_import<PBF16><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, in, field);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int field_import_unit(qed3_dirac_s* d, S64* field, const double* in_ref, double* part, double* nrm, cudaStream_t st) {
  const long long n = 4LL * d->Ns;
  const int parts = std::min(kNormParts, nblk(n));
  k_norm_part<<<parts, 256, 0, st>>>(n, in_ref, part);
  k_import_unit<<<nblk(d->Ns), 256, 0, st>>>(d->Ns, d->lat->dev.perm, reinterpret_cast<const S64*>(in_ref), part,
                                              parts, field, nrm);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int field_export_scaled(qed3_dirac_s* d, double* out_ref, const S64* field, const double* nrm, cudaStream_t st) {
  k_export_scaled<<<nblk(d->Ns), 256, 0, st>>>(d->Ns, d->lat->dev.perm, field, nrm, reinterpret_cast<S64*>(out_ref));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int field_export(qed3_dirac_s* d, int prec, double* out_ref, const void* field, int nrhs, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  const int g = nblk(d->Ns);
  S64* out = reinterpret_cast<S64*>(out_ref);
  if (prec == QED3_PREC_F64) k_export<P64><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, field, out);
  else if (prec == QED3_PREC_F32) k_export<P32><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, field, out);
  else k_export<PBF16><<<g, 256, 0, st>>>(d->Ns, nrhs, D.perm, field, out);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int dirac_apply_field(qed3_dirac_s* d, int op, int prec, void* out, const void* in, int nrhs, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  const int Ns = d->Ns;
  const int g = nblk(Ns);
  if (op != QED3_OP_D && op != QED3_OP_DDAG) return fail(QED3_ERR_ARG, "field apply supports D and D^dagger");
  const bool dag = op == QED3_OP_DDAG;
  if (prec == QED3_PREC_F64)
    k_apply64<<<g, 256, 0, st>>>(Ns, nrhs, D.nbr, dag ? d->Hd : d->H, d->diag, reinterpret_cast<const S64*>(in),
                                 reinterpret_cast<S64*>(out));
  else if (prec == QED3_PREC_F32)
    k_apply32<P32><<<g, 256, 0, st>>>(Ns, nrhs, D.nbr, dag ? d->Hd32 : d->H32, d->diag32,
                                      reinterpret_cast<const float4*>(in), reinterpret_cast<float4*>(out));
  else
    k_apply32<PBF16><<<g, 256, 0, st>>>(Ns, nrhs, D.nbr, dag ? d->Hd32 : d->H32, d->diag32,
                                        reinterpret_cast<const uint2*>(in), reinterpret_cast<uint2*>(out));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int dirac_apply32_blocks(qed3_dirac_s* d, const M32* H, void* out, const void* in, int nrhs, cudaStream_t st) {
  const DeviceLattice& D = d->lat->dev;
  k_apply32<P32><<<nblk(d->Ns), 256, 0, st>>>(d->Ns, nrhs, D.nbr, H, d->diag32, reinterpret_cast<const float4*>(in),
                                              reinterpret_cast<float4*>(out));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

}  // namespace qed3
