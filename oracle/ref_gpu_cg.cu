// The reference's GPU CG, restated for the benchmark's "reference design"
// baseline (bench.py `ref_gpu_baseline`).  Test and baseline infrastructure:
// nothing in the qed3_gb300 product calls it.  It is compiled for sm_103a
// like the product, so it shows what the reference's algorithm gives on the
// same GPU.
//
// What it restates, step for step:
//   * the CSR SpMV kernel `mult` (src/both_3d/gpu_header.h:102-117): one
//     thread per row, 256-thread blocks, (N + 256) / 256 blocks, the row's
//     result accumulated through res[i] in global memory;
//   * `Taxpy` (src/both_3d/gpu_header.h:126-130): d_res = a x + y, a by value;
//   * MatPoly::on_gpu (src/both_3d/matpoly.h:62-84) for the single product
//     chain {D, D^dagger}: two cudaMalloc, a memset, two D2D copies, the
//     products with a D2D copy after each, one Taxpy with coefficient 1, two
//     cudaFree -- per call;
//   * MatPoly::dot / dot2self (src/both_3d/matpoly.h:129-162):
//     cublasZdotc with the result returned to the host;
//   * MatPoly::solve (src/both_3d/matpoly.h:186-267), the host-vector form:
//     cudaMalloc x and r, copy b to the device, x0 = 0, q = 0, p = r = b,
//     complex alpha = mu / <p, q>, stop when |r|^2 < tol^2 |b|^2 on the
//     recursive residual, then copy x back and free.
// Setup (DWDevice: CSR arrays uploaded once) is outside the timed solves.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include <cublas_v2.h>
#include <cuComplex.h>
#include <cuda_runtime.h>

namespace {
using CuC = cuDoubleComplex;

__global__ void k_ref_mult(CuC* res, const CuC* v, const CuC* val, const int* cols, const int* rows, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    res[i] = make_cuDoubleComplex(0.0, 0.0);
    const int row_start = rows[i];
    const int row_end = rows[i + 1];
    for (int jj = row_start; jj < row_end; jj++) res[i] = cuCadd(res[i], cuCmul(val[jj], v[cols[jj]]));
  }
}

__global__ void k_ref_taxpy(CuC* d_res, const CuC a, const CuC* d_x, const CuC* d_y, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) d_res[i] = cuCadd(cuCmul(a, d_x[i]), d_y[i]);
}

struct Csr {
  int* rows = nullptr;
  int* cols = nullptr;
  CuC* val = nullptr;
};

#define RCHECK(x)                                                                     \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess) {                                                          \
      std::fprintf(stderr, "ref_gpu_cg: %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
      return -1;                                                                      \
    }                                                                                 \
  } while (0)
#define BCHECK(x)                                   \
  do {                                              \
    if ((x) != CUBLAS_STATUS_SUCCESS) return -1;    \
  } while (0)

struct Solver {
  int N = 0;
  Csr D, DH;
  cublasHandle_t h = nullptr;
  int blocks() const { return (N + 256) / 256; }

  int mult(const Csr& M, CuC* res, const CuC* v) const {
    k_ref_mult<<<blocks(), 256>>>(res, v, M.val, M.cols, M.rows, N);
    RCHECK(cudaGetLastError());
    return 0;
  }
  // MatPoly::on_gpu for the chain {D, D^dagger} with coefficient 1
  int on_gpu(CuC* d_v, const CuC* d_v0) const {
    CuC *d_tmp, *d_Mv0;
    const size_t bytes = size_t(N) * sizeof(CuC);
    RCHECK(cudaMalloc(&d_tmp, bytes));
    RCHECK(cudaMalloc(&d_Mv0, bytes));
    RCHECK(cudaMemset(d_v, 0, bytes));
    RCHECK(cudaMemcpy(d_tmp, d_v0, bytes, cudaMemcpyDeviceToDevice));
    RCHECK(cudaMemcpy(d_Mv0, d_v0, bytes, cudaMemcpyDeviceToDevice));
    if (mult(D, d_Mv0, d_tmp)) return -1;
    RCHECK(cudaMemcpy(d_tmp, d_Mv0, bytes, cudaMemcpyDeviceToDevice));
    if (mult(DH, d_Mv0, d_tmp)) return -1;
    RCHECK(cudaMemcpy(d_tmp, d_Mv0, bytes, cudaMemcpyDeviceToDevice));
    k_ref_taxpy<<<blocks(), 256>>>(d_v, make_cuDoubleComplex(1.0, 0.0), d_Mv0, d_v, N);
    RCHECK(cudaGetLastError());
    RCHECK(cudaFree(d_tmp));
    RCHECK(cudaFree(d_Mv0));
    return 0;
  }
  int dot(CuC* out, const CuC* x, const CuC* y) const {
    BCHECK(cublasZdotc(h, N, x, 1, y, 1, out));
    return 0;
  }
  // MatPoly::solve(d_x, d_b, tol, maxiter); returns the iteration count
  int solve_dev(CuC* d_x, const CuC* d_b, double tol, int maxiter) const {
    CuC *d_p, *d_q, *d_r;
    const size_t bytes = size_t(N) * sizeof(CuC);
    RCHECK(cudaMalloc(&d_p, bytes));
    RCHECK(cudaMalloc(&d_q, bytes));
    RCHECK(cudaMalloc(&d_r, bytes));
    RCHECK(cudaMemset(d_x, 0, bytes));
    RCHECK(cudaMemset(d_q, 0, bytes));
    RCHECK(cudaMemcpy(d_r, d_b, bytes, cudaMemcpyDeviceToDevice));
    RCHECK(cudaMemcpy(d_p, d_r, bytes, cudaMemcpyDeviceToDevice));
    CuC z;
    if (dot(&z, d_r, d_r)) return -1;
    double mu = cuCreal(z), mu_old = mu;
    if (dot(&z, d_r, d_r)) return -1;
    const double mu_crit = tol * tol * cuCreal(z);
    int k = 0, iters = 0;
    if (!(mu < mu_crit)) {
      for (; k < maxiter; ++k) {
        if (on_gpu(d_q, d_p)) return -1;
        CuC gam;
        if (dot(&gam, d_p, d_q)) return -1;
        const CuC al = cuCdiv(make_cuDoubleComplex(mu, 0.0), gam);
        k_ref_taxpy<<<blocks(), 256>>>(d_x, al, d_p, d_x, N);
        k_ref_taxpy<<<blocks(), 256>>>(d_r, make_cuDoubleComplex(-cuCreal(al), -cuCimag(al)), d_q, d_r, N);
        if (dot(&z, d_r, d_r)) return -1;
        mu = cuCreal(z);
        if (mu < mu_crit || std::isnan(mu)) break;
        const CuC bet = make_cuDoubleComplex(mu / mu_old, 0.0);
        mu_old = mu;
        k_ref_taxpy<<<blocks(), 256>>>(d_p, bet, d_p, d_r, N);
      }
      iters = k < maxiter ? k + 1 : k;
    }
    RCHECK(cudaFree(d_r));
    RCHECK(cudaFree(d_p));
    RCHECK(cudaFree(d_q));
    return iters;
  }
};

int upload(Csr& M, int N, int nnz, const int* rows, const int* cols, const double* val) {
  RCHECK(cudaMalloc(&M.rows, sizeof(int) * (N + 1)));
  RCHECK(cudaMalloc(&M.cols, sizeof(int) * nnz));
  RCHECK(cudaMalloc(&M.val, sizeof(CuC) * nnz));
  RCHECK(cudaMemcpy(M.rows, rows, sizeof(int) * (N + 1), cudaMemcpyHostToDevice));
  RCHECK(cudaMemcpy(M.cols, cols, sizeof(int) * nnz, cudaMemcpyHostToDevice));
  RCHECK(cudaMemcpy(M.val, val, sizeof(CuC) * nnz, cudaMemcpyHostToDevice));
  return 0;
}
void release(Csr& M) {
  cudaFree(M.rows);
  cudaFree(M.cols);
  cudaFree(M.val);
}
}  // namespace

// Solves (D^dag D) x = b `reps` times through the host-vector MatPoly::solve
// (after `warmup` untimed solves) with D and D^dag given as CSR arrays (values
// complex interleaved).  ms_out[r] = wall time of solve r (host copies
// included, as the reference's solve makes them); x_host receives the last
// solution.  Returns the iteration count of the last solve, or -1 on a CUDA
// or cuBLAS error.
extern "C" int refgpu_cg(int N, int nnz, const int* rows, const int* cols, const double* val, const int* rowsT,
                         const int* colsT, const double* valH, const double* b_host, double* x_host, double tol,
                         int maxiter, int warmup, int reps, double* ms_out) {
  Solver s;
  s.N = N;
  if (upload(s.D, N, nnz, rows, cols, val) || upload(s.DH, N, nnz, rowsT, colsT, valH)) return -1;
  if (cublasCreate(&s.h) != CUBLAS_STATUS_SUCCESS) return -1;
  const size_t bytes = size_t(N) * sizeof(CuC);
  int iters = -1;
  for (int r = 0; r < warmup + reps; r++) {
    const auto t0 = std::chrono::steady_clock::now();
    CuC *d_x, *d_r;
    RCHECK(cudaMalloc(&d_x, bytes));
    RCHECK(cudaMalloc(&d_r, bytes));
    RCHECK(cudaMemcpy(d_r, b_host, bytes, cudaMemcpyHostToDevice));
    iters = s.solve_dev(d_x, d_r, tol, maxiter);
    RCHECK(cudaMemcpy(x_host, d_x, bytes, cudaMemcpyDeviceToHost));
    RCHECK(cudaFree(d_x));
    RCHECK(cudaFree(d_r));
    if (iters < 0) break;
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r >= warmup) ms_out[r - warmup] = ms;
  }
  cublasDestroy(s.h);
  release(s.D);
  release(s.DH);
  return iters;
}
