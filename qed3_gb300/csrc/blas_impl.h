// FP64 vector helpers (blas.cu).
#pragma once

#include <cuda_runtime.h>

namespace qed3 {
constexpr int kMaxPoles = 64;
struct PoleCoef {
  double c[kMaxPoles];
};
int vec_axpby(long long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t st);
// out = a x + y over nc complex elements, a = are + i aim
int vec_zaxpy(long long nc, double are, double aim, const double* x, const double* y, double* out, cudaStream_t st);
int vec_pole_sum(long long n, int np, const double* coef, const double* Z, const double* x0, double* y,
                 cudaStream_t st);
// conj(x) . y over nc complex elements; part: device scratch of >= 2048 doubles
int vec_zdot(long long nc, const double* x, const double* y, double* part, double* re, double* im, cudaStream_t st);
}  // namespace qed3
