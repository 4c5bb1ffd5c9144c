// FP64 vector kernels on reference-order complex vectors (the Taxpy_gen /
// cublasZdotc work of src/dual/gpu_header.h:120-143, src/dual/matpoly.h:129-183)
// used by the overlap driver.  Dot products are deterministic: fixed block
// partials summed in order on the host.

#include <vector>

#include "blas_impl.h"
#include "device.cuh"
#include "handles.h"

namespace qed3 {

static inline int nblk(long long n, int t = 256) { return int((n + t - 1) / t); }

// out = a x + b y  (n doubles; real coefficients)
__global__ void k_axpby(long long n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                        double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a * x[i] + b * y[i];
}

// out = a x + y over complex elements (complex a; out may alias x or y)
__global__ void k_zaxpy(long long nc, double2 a, const double2* x, const double2* y, double2* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const double2 u = x[i], v = y[i];
  out[i] = make_double2(fma(a.x, u.x, fma(-a.y, u.y, v.x)), fma(a.x, u.y, fma(a.y, u.x, v.y)));
}

// y = x0 + sum_m c_m Z_m, Z stored as np consecutive vectors of n doubles
__global__ void k_pole_sum(long long n, int np, PoleCoef c, const double* __restrict__ Z,
                           const double* __restrict__ x0, double* __restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = x0[i];
  for (int m = 0; m < np; m++) acc += c.c[m] * Z[size_t(m) * n + i];
  y[i] = acc;
}

// partial sums of conj(x) y over complex elements
__global__ void k_zdot_part(long long nc, const double2* __restrict__ x, const double2* __restrict__ y,
                            double* __restrict__ part) {
  __shared__ double sh[64];
  double v[2] = {0.0, 0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    const double2 a = x[i], b = y[i];
    v[0] += a.x * b.x + a.y * b.y;
    v[1] += a.x * b.y - a.y * b.x;
  }
  block_sum<2>(v, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = v[0];
    part[2 * blockIdx.x + 1] = v[1];
  }
}

int vec_axpby(long long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t st) {
  k_axpby<<<nblk(n), 256, 0, st>>>(n, a, x, b, y, out);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int vec_zaxpy(long long nc, double are, double aim, const double* x, const double* y, double* out, cudaStream_t st) {
  k_zaxpy<<<nblk(nc), 256, 0, st>>>(nc, make_double2(are, aim), reinterpret_cast<const double2*>(x),
                                    reinterpret_cast<const double2*>(y), reinterpret_cast<double2*>(out));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int vec_pole_sum(long long n, int np, const double* coef, const double* Z, const double* x0, double* y,
                 cudaStream_t st) {
  if (np > kMaxPoles) return fail(QED3_ERR_ARG, "too many poles");
  PoleCoef c{};
  for (int m = 0; m < np; m++) c.c[m] = coef[m];
  k_pole_sum<<<nblk(n), 256, 0, st>>>(n, np, c, Z, x0, y);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int vec_zdot(long long nc, const double* x, const double* y, double* part, double* re, double* im, cudaStream_t st) {
  const int g = std::min(1024, std::max(1, nblk(nc)));
  k_zdot_part<<<g, 256, 0, st>>>(nc, reinterpret_cast<const double2*>(x), reinterpret_cast<const double2*>(y), part);
  QED3_CUDA_TRY(cudaGetLastError());
  std::vector<double> h(2 * size_t(g));
  QED3_CUDA_TRY(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  double a = 0, b = 0;
  for (int i = 0; i < g; i++) {
    a += h[2 * i];
    b += h[2 * i + 1];
  }
  *re = a;
  if (im) *im = b;
  return QED3_OK;
}

}  // namespace qed3
