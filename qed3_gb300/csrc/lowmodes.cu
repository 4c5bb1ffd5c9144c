// Low eigenmodes of a hermitian positive semidefinite operator on
// reference-order complex vectors: Lanczos with full reorthogonalisation.
//
// Used for the low-mode projection of the overlap's sign function: the
// reference's Overlap (src/both_3d/overlap.h:137-390) approximates
// sign(H) by one Zolotarev rational function on [lambda_min, lambda_max] of
// |H|, so a few near-zero modes of H_W = gamma5 D_W set k = lambda_min /
// lambda_max (1.9e-4 at n=32, beta=1.4, M5=-1) and with it the condition of
// every pole solve (1/k^2 ~ 3e7) and the accuracy of 20 poles (~1e-8).
// Treating the nev lowest modes of H_W exactly raises k to the (nev+1)-th
// (4.8e-3 for nev=20 there).
//
// Algorithm: the Lanczos three-term recurrence on A (FP64, one product per
// step), every new vector orthogonalised against all previous ones by
// classical Gram-Schmidt (a second pass when the first removed more than
// 30 % of the norm), so the basis V stays orthonormal to rounding.  The
// nev+1 smallest eigenvalues of the tridiagonal T come from Sturm bisection,
// their eigenvectors s from inverse iteration; a Ritz pair has converged when
// beta_j |s_j| <= tol * theta_max.  Ritz vectors y = V s are formed on the
// device.  lanczos_lowmodes() then recomputes every residual explicitly.

#include <algorithm>
#include <cmath>
#include <functional>
#include <random>
#include <vector>

#include "blas_impl.h"
#include "device.cuh"
#include "handles.h"
#include "lowmodes_impl.h"

namespace qed3 {

namespace {
constexpr int kTileC = 2048;  // complex entries per dot tile (256 threads x 8)
constexpr int kJB = 16;       // basis vectors per dot block

// part[j][tile] = sum over the tile of conj(V_j) w, for j in [jb, jb + kJB)
__global__ void k_gs_dots(long long nc, int m, const double2* __restrict__ V, const double2* __restrict__ w,
                          double* __restrict__ part, int ntiles) {
  __shared__ double sh[64];
  const int tile = blockIdx.x;
  const int j0 = blockIdx.y * kJB;
  double2 wl[kTileC / 256];
#pragma unroll
  for (int k = 0; k < kTileC / 256; k++) {
    const long long e = (long long)tile * kTileC + k * 256 + threadIdx.x;
    wl[k] = e < nc ? w[e] : make_double2(0.0, 0.0);
  }
  for (int j = j0; j < min(m, j0 + kJB); j++) {
    const double2* Vj = V + (size_t)j * nc;
    double v[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < kTileC / 256; k++) {
      const long long e = (long long)tile * kTileC + k * 256 + threadIdx.x;
      if (e < nc) {
        const double2 a = Vj[e];
        v[0] += a.x * wl[k].x + a.y * wl[k].y;
        v[1] += a.x * wl[k].y - a.y * wl[k].x;
      }
    }
    block_sum<2>(v, sh);
    if (threadIdx.x == 0) {
      part[2 * ((size_t)j * ntiles + tile)] = v[0];
      part[2 * ((size_t)j * ntiles + tile) + 1] = v[1];
    }
  }
}

// c_j = sum over tiles in order (deterministic)
__global__ void k_gs_sum(int m, int ntiles, const double* __restrict__ part, double2* __restrict__ c) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double re = 0.0, im = 0.0;
  for (int t = 0; t < ntiles; t++) {
    re += part[2 * ((size_t)j * ntiles + t)];
    im += part[2 * ((size_t)j * ntiles + t) + 1];
  }
  c[j] = make_double2(re, im);
}

// w -= sum_j c_j V_j
__global__ void k_gs_update(long long nc, int m, const double2* __restrict__ V, const double2* __restrict__ c,
                            double2* __restrict__ w) {
  __shared__ double2 cs[1024];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double2 acc = make_double2(0.0, 0.0);
  for (int j0 = 0; j0 < m; j0 += 1024) {
    const int cnt = min(1024, m - j0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) cs[k] = c[j0 + k];
    __syncthreads();
    if (e < nc)
      for (int k = 0; k < cnt; k++) {
        const double2 a = V[(size_t)(j0 + k) * nc + e], cc = cs[k];
        acc.x += cc.x * a.x - cc.y * a.y;
        acc.y += cc.x * a.y + cc.y * a.x;
      }
  }
  if (e < nc) {
    const double2 x = w[e];
    w[e] = make_double2(x.x - acc.x, x.y - acc.y);
  }
}

// Y_i = sum_j S[j][i] V_j for i in [0, cnt) (S complex, row-major [m][ldS], i offset i0)
constexpr int kCombine = 8;
__global__ void k_combine(long long nc, int m, const double2* __restrict__ V, const double2* __restrict__ S, int ldS,
                          int i0, int cnt, double2* __restrict__ Y) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nc) return;
  double2 acc[kCombine];
#pragma unroll
  for (int i = 0; i < kCombine; i++) acc[i] = make_double2(0.0, 0.0);
  for (int j = 0; j < m; j++) {
    const double2 a = V[(size_t)j * nc + e];
#pragma unroll
    for (int i = 0; i < kCombine; i++) {
      if (i < cnt) {
        const double2 s = S[(size_t)j * ldS + i0 + i];
        acc[i].x += s.x * a.x - s.y * a.y;
        acc[i].y += s.x * a.y + s.y * a.x;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < kCombine; i++)
    if (i < cnt) Y[(size_t)(i0 + i) * nc + e] = acc[i];
}

int nblocks(long long n, int t) { return int((n + t - 1) / t); }

// ---- host: symmetric tridiagonal T (a diagonal, b off-diagonal) -----------------------------
int sturm(const std::vector<double>& a, const std::vector<double>& b, int m, double x) {
  int count = 0;
  double q = a[0] - x;
  if (q < 0) count++;
  for (int i = 1; i < m; i++) {
    const double qq = q != 0.0 ? q : 1e-300;
    q = a[i] - x - b[i - 1] * b[i - 1] / qq;
    if (q < 0) count++;
  }
  return count;
}

double tri_eig(const std::vector<double>& a, const std::vector<double>& b, int m, int k) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; i++) {
    const double r = (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i < m - 1 ? std::abs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double scale = std::max(std::abs(lo), std::abs(hi));
  for (int it = 0; it < 200 && hi - lo > 2e-16 * scale; it++) {
    const double mid = 0.5 * (lo + hi);
    if (sturm(a, b, m, mid) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// Solves (T - theta) x = y in place: LU with partial pivoting of the
// tridiagonal (the row-exchange scheme of LAPACK's dgttrf / dgtts2, written
// out here); a vanishing pivot is replaced by a tiny one, as inverse
// iteration wants.
void tri_solve(const std::vector<double>& a, const std::vector<double>& b, int m, double theta, std::vector<double>& y) {
  std::vector<double> D(m), DL(m, 0.0), DU(m, 0.0), DU2(m, 0.0);
  std::vector<char> sw(m, 0);
  double scale = 0;
  for (int i = 0; i < m; i++) {
    D[i] = a[i] - theta;
    if (i < m - 1) DL[i] = DU[i] = b[i];
    scale = std::max(scale, std::abs(D[i]) + (i < m - 1 ? std::abs(b[i]) : 0.0));
  }
  const double tiny = std::max(scale * 1e-300, 1e-300) + scale * 1e-17;
  for (int i = 0; i < m - 1; i++) {
    if (std::abs(D[i]) >= std::abs(DL[i])) {
      if (D[i] == 0.0) D[i] = tiny;
      const double f = DL[i] / D[i];
      DL[i] = f;
      D[i + 1] -= f * DU[i];
    } else {
      const double f = D[i] / DL[i];
      D[i] = DL[i];
      DL[i] = f;
      const double t = DU[i];
      DU[i] = D[i + 1];
      D[i + 1] = t - f * D[i + 1];
      if (i < m - 2) {
        DU2[i] = DU[i + 1];
        DU[i + 1] = -f * DU[i + 1];
      }
      sw[i] = 1;
    }
  }
  if (D[m - 1] == 0.0) D[m - 1] = tiny;
  for (int i = 0; i < m - 1; i++) {
    if (!sw[i]) {
      y[i + 1] -= DL[i] * y[i];
    } else {
      const double t = y[i];
      y[i] = y[i + 1];
      y[i + 1] = t - DL[i] * y[i];
    }
  }
  y[m - 1] /= D[m - 1];
  if (m > 1) y[m - 2] = (y[m - 2] - DU[m - 2] * y[m - 1]) / D[m - 2];
  for (int i = m - 3; i >= 0; i--) y[i] = (y[i] - DU[i] * y[i + 1] - DU2[i] * y[i + 2]) / D[i];
}

// Eigenvectors of T for the given (ascending) eigenvalues by inverse
// iteration, orthogonalised within clusters of close eigenvalues.
void tri_vectors(const std::vector<double>& a, const std::vector<double>& b, int m, const std::vector<double>& th,
                 std::vector<std::vector<double>>& S) {
  std::mt19937_64 gen(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const double scale = std::max(std::abs(th.front()), std::abs(th.back())) + 1e-300;
  S.assign(th.size(), std::vector<double>(m));
  for (size_t k = 0; k < th.size(); k++) {
    std::vector<double>& s = S[k];
    for (auto& v : s) v = U(gen);
    for (int it = 0; it < 4; it++) {
      tri_solve(a, b, m, th[k], s);
      for (size_t q = 0; q < k; q++) {  // orthogonal to the cluster's earlier vectors
        if (std::abs(th[q] - th[k]) > 1e-7 * scale) continue;
        double dp = 0;
        for (int i = 0; i < m; i++) dp += S[q][i] * s[i];
        for (int i = 0; i < m; i++) s[i] -= dp * S[q][i];
      }
      double nrm = 0;
      for (double v : s) nrm += v * v;
      nrm = std::sqrt(nrm);
      for (auto& v : s) v /= nrm;
    }
  }
}
}  // namespace

// Lanczos with full reorthogonalisation on a hermitian `apply`: the nv Ritz
// pairs at the low end (largest = false) or the high end (largest = true),
// converged to beta |s_last| <= tol * max|theta| (or after maxsteps when
// require = false).  *vec_out: device, nv vectors; theta in the order of the
// end (ascending for the low end, descending for the high end); *extreme =
// the Ritz value at the opposite end.
static int lanczos_core(long long nd, const std::function<int(double*, const double*)>& apply, int nv, bool largest,
                        double tol, int maxsteps, bool require, double** vec_out, std::vector<double>& theta,
                        double* extreme, int* steps_used, cudaStream_t st, bool* conv_out = nullptr) {
  const int nev = nv - 1;
  if (nv < 1 || maxsteps < nv + 2 || !(tol > 0)) return fail(QED3_ERR_ARG, "low modes: bad Lanczos arguments");
  const long long nc = nd / 2;
  if (maxsteps > nc) maxsteps = int(nc);
  const int ntiles = int((nc + kTileC - 1) / kTileC);
  double *V = nullptr, *w = nullptr, *part = nullptr, *cj = nullptr, *gsp = nullptr;
  size_t vbytes = size_t(maxsteps + 1) * nd * sizeof(double);
  auto cleanup = [&]() {
    if (V) cudaFree(V);
    if (w) cudaFree(w);
    if (part) cudaFree(part);
    if (cj) cudaFree(cj);
    if (gsp) cudaFree(gsp);
  };
  if (cudaMalloc(&V, vbytes) != cudaSuccess || cudaMalloc(&w, nd * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&part, 2048 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&cj, size_t(maxsteps + 1) * 2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&gsp, size_t(maxsteps + 1) * ntiles * 2 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
  }
  auto col = [&](int j) { return V + size_t(j) * nd; };
  auto body = [&]() -> int {
    std::vector<double> h(static_cast<size_t>(nd));
    std::mt19937_64 gen(20261204);
    std::normal_distribution<double> nrm;
    for (auto& x : h) x = nrm(gen);
    QED3_CUDA_TRY(cudaMemcpyAsync(col(0), h.data(), nd * sizeof(double), cudaMemcpyHostToDevice, st));
    double re = 0, im = 0;
    int e = vec_zdot(nc, col(0), col(0), part, &re, &im, st);
    if (e) return e;
    if ((e = vec_axpby(nd, 1.0 / std::sqrt(re), col(0), 0.0, col(0), col(0), st))) return e;
    std::vector<double> al, be;
    int j = 0, next_check = largest ? nev + 12 : std::max(2 * nev + 20, 60);
    bool done = false, conv = false;
    std::vector<double> th;
    std::vector<std::vector<double>> S;
    double tmax = 0;
    auto gs_pass = [&](int m) -> int {  // w -= V[0..m) (V^H w)
      dim3 g(ntiles, (m + kJB - 1) / kJB);
      k_gs_dots<<<g, 256, 0, st>>>(nc, m, reinterpret_cast<const double2*>(V), reinterpret_cast<const double2*>(w),
                                   gsp, ntiles);
      k_gs_sum<<<nblocks(m, 128), 128, 0, st>>>(m, ntiles, gsp, reinterpret_cast<double2*>(cj));
      k_gs_update<<<nblocks(nc, 256), 256, 0, st>>>(nc, m, reinterpret_cast<const double2*>(V),
                                                     reinterpret_cast<const double2*>(cj),
                                                     reinterpret_cast<double2*>(w));
      QED3_CUDA_TRY(cudaGetLastError());
      return QED3_OK;
    };
    for (; j < maxsteps && !done; j++) {
      if ((e = apply(w, col(j)))) return e;
      if ((e = vec_zdot(nc, col(j), w, part, &re, &im, st))) return e;
      al.push_back(re);  // real: A is hermitian
      double w0 = 0;
      if ((e = vec_zdot(nc, w, w, part, &w0, &im, st))) return e;
      if ((e = gs_pass(j + 1))) return e;  // removes alpha v_j, beta v_{j-1} and any drift
      double w1 = 0;
      if ((e = vec_zdot(nc, w, w, part, &w1, &im, st))) return e;
      if (w1 < 0.49 * w0) {
        if ((e = gs_pass(j + 1))) return e;
        if ((e = vec_zdot(nc, w, w, part, &w1, &im, st))) return e;
      }
      const double beta = std::sqrt(std::max(w1, 0.0));
      const int m = j + 1;
      const bool last = beta <= 1e-14 * std::sqrt(std::max(w0, 1e-300)) || m == maxsteps;
      if (m >= next_check || last) {
        next_check = m + (largest ? std::max(8, m / 10) : std::max(40, m / 8));
        if (m > nev) {
          th.assign(nev + 1, 0.0);
          for (int k = 0; k <= nev; k++) th[k] = tri_eig(al, be, m, largest ? m - 1 - k : k);
          tmax = tri_eig(al, be, m, largest ? 0 : m - 1);
          if (largest) {  // inverse iteration wants ascending order
            std::vector<double> asc(th.rbegin(), th.rend());
            tri_vectors(al, be, m, asc, S);
            std::reverse(S.begin(), S.end());
          } else {
            tri_vectors(al, be, m, th, S);
          }
          double worst = 0;
          const double scale = std::max(std::abs(tmax), std::abs(th[0]));
          for (int k = 0; k <= nev; k++) worst = std::max(worst, beta * std::abs(S[k][m - 1]));
          conv = worst <= tol * scale;
          if (conv || last) done = true;
        }
      }
      if (!done) {
        be.push_back(beta);
        if ((e = vec_axpby(nd, 1.0 / beta, w, 0.0, w, col(j + 1), st))) return e;
      }
    }
    const int m = int(al.size());
    if (int(th.size()) != nev + 1) return fail(QED3_ERR_NOCONV, "low modes: Lanczos ended before nev + 1 steps");
    if (require && !conv) return fail(QED3_ERR_NOCONV, "low modes: Lanczos did not converge in maxsteps");
    const int nvec = nev + 1;
    // Ritz vectors: Y_i = V S_i
    double* Y = nullptr;
    if (cudaMalloc(&Y, size_t(nvec) * nd * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
    }
    std::vector<double> Sh(size_t(m) * nvec * 2, 0.0);  // complex [m][nvec]
    for (int jj = 0; jj < m; jj++)
      for (int i = 0; i < nvec; i++) Sh[2 * (size_t(jj) * nvec + i)] = S[i][jj];
    double* Sd = nullptr;
    if (cudaMalloc(&Sd, Sh.size() * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(Y);
      return fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
    }
    int rc = QED3_OK;
    if (cudaMemcpyAsync(Sd, Sh.data(), Sh.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
      rc = fail(QED3_ERR_CUDA, "low modes: copy failed");
    for (int i0 = 0; i0 < nvec && !rc; i0 += kCombine) {
      k_combine<<<nblocks(nc, 256), 256, 0, st>>>(nc, m, reinterpret_cast<const double2*>(V),
                                                   reinterpret_cast<const double2*>(Sd), nvec, i0,
                                                   std::min(kCombine, nvec - i0), reinterpret_cast<double2*>(Y));
      if (cudaGetLastError() != cudaSuccess) rc = fail(QED3_ERR_CUDA, "low modes: combine failed");
    }
    cudaStreamSynchronize(st);
    cudaFree(Sd);
    if (rc) {
      cudaFree(Y);
      return rc;
    }
    theta = th;
    *extreme = tmax;
    *steps_used = m;
    *vec_out = Y;
    if (conv_out) *conv_out = conv;
    return QED3_OK;
  };
  const int rc = body();
  cleanup();
  return rc;
}

// Chebyshev filter q(A) v = T_d((a + b - 2 A) / (b - a)) v: |q| <= 1 on [a, b],
// growing fast below a, so the low end of A becomes the well separated high
// end of q(A).  out = c1 x + c2 y + c3 z
__global__ void k_lin3(long long n, double c1, const double* __restrict__ x, double c2, const double* __restrict__ y,
                       double c3, const double* __restrict__ z, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = c1 * x[i] + c2 * y[i] + c3 * z[i];
}

// The nev smallest eigenpairs of the hermitian PSD `apply` (see the header):
// a short pilot Lanczos gives an upper bound a of the (nev+1)-th eigenvalue
// and b of the largest; Lanczos on the Chebyshev-filtered q(A) (degree
// ~ 2.5 sqrt(b / a)) then converges the nev + 1 largest q, i.e. the nev + 1
// smallest eigenvalues of A, in few steps even when they are 1e-7 of b apart.
// Their eigenvalues are the Rayleigh quotients with A; explicit residuals.
int lanczos_lowmodes(long long nd, const std::function<int(double*, const double*)>& apply, int nev, double tol,
                     int maxsteps, double** vec_out, std::vector<double>& theta, double* theta_next,
                     double* theta_max, double* max_res, int* steps_used, cudaStream_t st) {
  if (nev < 1 || !(tol > 0) || maxsteps < 2 * nev + 20) return fail(QED3_ERR_ARG, "low modes: need nev >= 1, tol > 0, maxsteps >= 2 nev + 20");
  const long long nc = nd / 2;
  // pilot: a short unconverged Lanczos on A
  double* P = nullptr;
  std::vector<double> pth;
  double pmax = 0;
  int psteps = 0;
  int rc = lanczos_core(nd, apply, nev + 1, false, 1e-300, std::min<long long>(maxsteps, std::min<long long>(nc, 3LL * nev + 80)),
                        false, &P, pth, &pmax, &psteps, st);
  if (P) cudaFree(P);
  if (rc) return rc;
  double b = 1.02 * pmax, a = 1.5 * pth[nev];
  double* buf = nullptr;
  if (cudaMalloc(&buf, 4 * size_t(nd) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
  }
  int total_steps = psteps;
  double* Y = nullptr;
  std::vector<double> th_out;
  double res_out = 0, next_out = 0;
  for (int attempt = 0; attempt < 10; attempt++) {
    if (!(a > 0 && a < b)) {
      rc = fail(QED3_ERR_NOCONV, "low modes: no spectral gap for the filter");
      break;
    }
    const int deg = std::min(2000, std::max(8, int(std::ceil(2.5 / std::sqrt(a / b)))));
    const double al = -2.0 / (b - a), be = (a + b) / (b - a);
    double *T0 = buf, *T1 = buf + nd, *T2 = buf + 2 * nd, *AT = buf + 3 * nd;
    auto filt = [&](double* out, const double* v) -> int {
      int e;
      QED3_CUDA_TRY(cudaMemcpyAsync(T0, v, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if ((e = apply(AT, T0))) return e;
      k_lin3<<<nblocks(nd, 256), 256, 0, st>>>(nd, al, AT, be, T0, 0.0, T0, T1);  // T1 = L v
      double *pm = T0, *pc = T1, *pn = T2;
      for (int k = 1; k < deg; k++) {
        if ((e = apply(AT, pc))) return e;
        k_lin3<<<nblocks(nd, 256), 256, 0, st>>>(nd, 2.0 * al, AT, 2.0 * be, pc, -1.0, pm, pn);
        double* t = pm;
        pm = pc;
        pc = pn;
        pn = t;
      }
      QED3_CUDA_TRY(cudaGetLastError());
      QED3_CUDA_TRY(cudaMemcpyAsync(out, pc, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
      return QED3_OK;
    };
    std::vector<double> qth;
    double qmin = 0;
    int qsteps = 0;
    double* Yq = nullptr;
    bool conv = false;
    rc = lanczos_core(nd, filt, nev + 1, true, tol, std::min(maxsteps, 8 * (nev + 1) + 200), false, &Yq, qth, &qmin,
                      &qsteps, st, &conv);
    total_steps += qsteps * deg;
    if (rc) {
      if (Yq) cudaFree(Yq);
      break;
    }
    if (!conv) {
      // Too many modes amplified for the step budget: move the cut down to an
      // upper bound of the (nev+1)-th eigenvalue read off the filtered Ritz
      // values (a Ritz value of q(A) is a lower bound of its eigenvalue, so the
      // inverse map x = (a + b - L (b - a)) / 2, L = cosh(acosh(q) / deg), bounds
      // the eigenvalue of A from above), at least halving it.
      cudaFree(Yq);
      double anew = 0.5 * a;
      if (qth[nev] > 1.0) {
        const double L = std::cosh(std::acosh(qth[nev]) / deg);
        anew = std::min(anew, 1.5 * 0.5 * (a + b - L * (b - a)));
      }
      a = anew;
      rc = QED3_OK;
      continue;
    }
    // Rayleigh quotients and residuals with A, ascending
    std::vector<double> ray(nev + 1), res(nev + 1);
    double* w = AT;
    for (int i = 0; i <= nev && !rc; i++) {
      double* yi = Yq + size_t(i) * nd;
      double re = 0, im = 0, r2 = 0;
      rc = apply(w, yi);
      if (!rc) rc = vec_zdot(nc, yi, w, T0, &re, &im, st);
      ray[i] = re;
      if (!rc) rc = vec_axpby(nd, 1.0, w, -re, yi, w, st);
      if (!rc) rc = vec_zdot(nc, w, w, T0, &r2, &im, st);
      res[i] = std::sqrt(std::max(r2, 0.0));
    }
    if (rc) {
      cudaFree(Yq);
      break;
    }
    const double top = *std::max_element(ray.begin(), ray.end());
    if (!(top < a)) {  // the (nev+1)-th mode is not inside the amplified range: widen it
      cudaFree(Yq);
      a *= 2.0;
      continue;
    }
    // order ascending in A (the filter is monotone below a, so this is the q order reversed)
    std::vector<int> idx(nev + 1);
    for (int i = 0; i <= nev; i++) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return ray[x] < ray[y]; });
    if (cudaMalloc(&Y, size_t(nev) * nd * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(Yq);
      rc = fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
      break;
    }
    th_out.assign(nev, 0.0);
    res_out = 0;
    for (int i = 0; i < nev; i++) {
      QED3_CUDA_TRY(cudaMemcpyAsync(Y + size_t(i) * nd, Yq + size_t(idx[i]) * nd, nd * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st));
      th_out[i] = ray[idx[i]];
      res_out = std::max(res_out, res[idx[i]]);
    }
    next_out = ray[idx[nev]];
    cudaStreamSynchronize(st);
    cudaFree(Yq);
    break;
  }
  cudaFree(buf);
  if (rc) return rc;
  if (!Y) return fail(QED3_ERR_NOCONV, "low modes: the filter range did not reach nev + 1 modes");
  theta = th_out;
  *theta_next = next_out;
  *theta_max = b;
  *max_res = res_out;
  *steps_used = total_steps;
  *vec_out = Y;
  return QED3_OK;
}

// ---- chirality ------------------------------------------------------------------------------
// gamma5 = sigma3 per site on reference-order two-spinors (complex index 2 x + s):
// c = 0: out = gamma5 in; c = +1 / -1: out = P_c in = (1 + c gamma5)/2 in
__global__ void k_chiral(long long nc, int c, const double2* __restrict__ in, double2* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const int g5 = (i & 1) ? -1 : 1;
  const double2 v = in[i];
  double f;
  if (c == 0) f = double(g5);
  else f = (g5 == c) ? 1.0 : 0.0;
  out[i] = make_double2(f * v.x, f * v.y);
}

int chiral(long long nd, int c, const double* in, double* out, cudaStream_t st) {
  const long long nc = nd / 2;
  k_chiral<<<nblocks(nc, 256), 256, 0, st>>>(nc, c, reinterpret_cast<const double2*>(in),
                                              reinterpret_cast<double2*>(out));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// ---- projections with a set of orthonormal complex vectors H[nev][nd] --------------------
// c = H^H v (host copy returned), then out = v - sum c_i H_i when out != nullptr
int modes_coeffs(long long nd, int nev, const double* H, const double* v, double* part, std::vector<double>& c,
                 cudaStream_t st) {
  c.assign(2 * size_t(nev), 0.0);
  for (int i = 0; i < nev; i++) {
    double re = 0, im = 0;
    int e = vec_zdot(nd / 2, H + size_t(i) * nd, v, part, &re, &im, st);
    if (e) return e;
    c[2 * i] = re;
    c[2 * i + 1] = im;
  }
  return QED3_OK;
}

// out = x + sum_i w_i H_i (complex weights w, host)
int modes_axpy(long long nd, int nev, const double* H, const std::vector<double>& wts, const double* x, double* out,
               cudaStream_t st) {
  int e = QED3_OK;
  if (out != x) QED3_CUDA_TRY(cudaMemcpyAsync(out, x, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  for (int i = 0; i < nev && !e; i++) e = vec_zaxpy(nd / 2, wts[2 * i], wts[2 * i + 1], H + size_t(i) * nd, out, out, st);
  return e;
}

// Y_i <- sum_j U[j][i] Y_j for a complex nev x nev matrix U (host, row-major [j][i])
int modes_rotate(long long nd, int nev, double* Y, const std::vector<double>& U, cudaStream_t st) {
  const long long nc = nd / 2;
  double *Sd = nullptr, *Out = nullptr;
  if (cudaMalloc(&Sd, U.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&Out, size_t(nev) * nd * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    if (Sd) cudaFree(Sd);
    return fail(QED3_ERR_NOMEM, "low modes: cudaMalloc failed");
  }
  int rc = QED3_OK;
  if (cudaMemcpyAsync(Sd, U.data(), U.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = fail(QED3_ERR_CUDA, "low modes: copy failed");
  for (int i0 = 0; i0 < nev && !rc; i0 += kCombine) {
    k_combine<<<nblocks(nc, 256), 256, 0, st>>>(nc, nev, reinterpret_cast<const double2*>(Y),
                                                 reinterpret_cast<const double2*>(Sd), nev, i0,
                                                 std::min(kCombine, nev - i0), reinterpret_cast<double2*>(Out));
    if (cudaGetLastError() != cudaSuccess) rc = fail(QED3_ERR_CUDA, "low modes: combine failed");
  }
  if (!rc && cudaMemcpyAsync(Y, Out, size_t(nev) * nd * sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    rc = fail(QED3_ERR_CUDA, "low modes: copy failed");
  cudaStreamSynchronize(st);
  cudaFree(Sd);
  cudaFree(Out);
  return rc;
}

// Eigen-decomposition of a complex hermitian n x n matrix G (row-major complex
// pairs) by cyclic Jacobi rotations on its real symmetric 2n x 2n form
// [[Re, -Im], [Im, Re]]; every eigenvalue appears twice there, with the
// vectors x and i x.  Returns the n eigenvalues (ascending) and complex
// eigenvectors U (row-major [component][index]).
void hermitian_eig(int n, const std::vector<double>& G, std::vector<double>& ev, std::vector<double>& U) {
  const int N = 2 * n;
  std::vector<double> M(size_t(N) * N), Q(size_t(N) * N, 0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const double re = G[2 * (size_t(i) * n + j)], im = G[2 * (size_t(i) * n + j) + 1];
      M[size_t(i) * N + j] = re;
      M[size_t(i + n) * N + j + n] = re;
      M[size_t(i) * N + j + n] = -im;
      M[size_t(i + n) * N + j] = im;
    }
  for (int i = 0; i < N; i++) Q[size_t(i) * N + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0, tot = 0;
    for (int p = 0; p < N; p++)
      for (int q = 0; q < N; q++) {
        tot += M[size_t(p) * N + q] * M[size_t(p) * N + q];
        if (p != q) off += M[size_t(p) * N + q] * M[size_t(p) * N + q];
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < N - 1; p++)
      for (int q = p + 1; q < N; q++) {
        const double apq = M[size_t(p) * N + q];
        if (std::abs(apq) < 1e-300) continue;
        const double app = M[size_t(p) * N + p], aqq = M[size_t(q) * N + q];
        const double tau = (aqq - app) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::abs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < N; k++) {  // columns p, q
          const double mkp = M[size_t(k) * N + p], mkq = M[size_t(k) * N + q];
          M[size_t(k) * N + p] = c * mkp - s * mkq;
          M[size_t(k) * N + q] = s * mkp + c * mkq;
        }
        for (int k = 0; k < N; k++) {  // rows p, q
          const double mpk = M[size_t(p) * N + k], mqk = M[size_t(q) * N + k];
          M[size_t(p) * N + k] = c * mpk - s * mqk;
          M[size_t(q) * N + k] = s * mpk + c * mqk;
        }
        for (int k = 0; k < N; k++) {
          const double qkp = Q[size_t(k) * N + p], qkq = Q[size_t(k) * N + q];
          Q[size_t(k) * N + p] = c * qkp - s * qkq;
          Q[size_t(k) * N + q] = s * qkp + c * qkq;
        }
      }
  }
  std::vector<int> order(N);
  for (int i = 0; i < N; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return M[size_t(a) * N + a] < M[size_t(b) * N + b]; });
  // pick n complex-orthonormal vectors from the 2n real ones, in ascending order
  ev.clear();
  U.assign(2 * size_t(n) * n, 0.0);
  std::vector<std::vector<double>> picked;  // complex vectors, 2n doubles each
  for (int idx : order) {
    if (int(picked.size()) == n) break;
    std::vector<double> x(2 * size_t(n));
    for (int i = 0; i < n; i++) {
      x[2 * i] = Q[size_t(i) * N + idx];
      x[2 * i + 1] = Q[size_t(i + n) * N + idx];
    }
    for (const auto& y : picked) {  // x -= <y, x> y
      double re = 0, im = 0;
      for (int i = 0; i < n; i++) {
        re += y[2 * i] * x[2 * i] + y[2 * i + 1] * x[2 * i + 1];
        im += y[2 * i] * x[2 * i + 1] - y[2 * i + 1] * x[2 * i];
      }
      for (int i = 0; i < n; i++) {
        x[2 * i] -= re * y[2 * i] - im * y[2 * i + 1];
        x[2 * i + 1] -= re * y[2 * i + 1] + im * y[2 * i];
      }
    }
    double nr = 0;
    for (double v : x) nr += v * v;
    if (nr < 0.25) continue;  // the partner (i x) of an already picked vector
    nr = std::sqrt(nr);
    for (auto& v : x) v /= nr;
    ev.push_back(M[size_t(idx) * N + idx]);
    picked.push_back(x);
  }
  for (int k = 0; k < int(picked.size()); k++)
    for (int i = 0; i < n; i++) {
      U[2 * (size_t(i) * n + k)] = picked[k][2 * i];
      U[2 * (size_t(i) * n + k) + 1] = picked[k][2 * i + 1];
    }
}

}  // namespace qed3
