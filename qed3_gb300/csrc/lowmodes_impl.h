// Low eigenmodes by Lanczos with full reorthogonalisation (lowmodes.cu).
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <vector>

namespace qed3 {
constexpr int kMaxLowModes = 256;
// The nev smallest eigenpairs of a hermitian PSD operator `apply` on complex
// vectors of nd doubles: *vec_out (device, cudaMalloc'ed, nev vectors back to
// back, orthonormal), theta (ascending), theta_next = the (nev+1)-th Ritz value,
// theta_max = the largest, max_res = max_i ||A y_i - theta_i y_i||.
int lanczos_lowmodes(long long nd, const std::function<int(double*, const double*)>& apply, int nev, double tol,
                     int maxsteps, double** vec_out, std::vector<double>& theta, double* theta_next,
                     double* theta_max, double* max_res, int* steps_used, cudaStream_t st);
// c = H^H v for nev orthonormal complex vectors H (host result, complex pairs)
int modes_coeffs(long long nd, int nev, const double* H, const double* v, double* part, std::vector<double>& c,
                 cudaStream_t st);
// out = x + sum_i w_i H_i (complex weights, host)
int modes_axpy(long long nd, int nev, const double* H, const std::vector<double>& wts, const double* x, double* out,
               cudaStream_t st);
// Y_i <- sum_j U[j][i] Y_j, U complex nev x nev (host, row-major)
int modes_rotate(long long nd, int nev, double* Y, const std::vector<double>& U, cudaStream_t st);
// c = 0: out = gamma5 in; c = +1 / -1: out = (1 + c gamma5)/2 in (reference-order two-spinors)
int chiral(long long nd, int c, const double* in, double* out, cudaStream_t st);
// complex hermitian n x n eigen-decomposition (host): ev ascending, U[i][k] = component i of vector k
void hermitian_eig(int n, const std::vector<double>& G, std::vector<double>& ev, std::vector<double>& U);
}  // namespace qed3
