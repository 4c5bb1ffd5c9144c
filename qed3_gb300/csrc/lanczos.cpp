// Extremal eigenvalues of D^dag D by the Lanczos recurrence, an alternative to
// the power / inverse-power iterations of Overlap::compute_lambda_max
// (src/both_3d/overlap.h:217-306), which need a CG solve per inverse
// iteration.  Plain three-term Lanczos in FP64 on the device (one D^dag D
// product and two inner products per step, no reorthogonalisation: lost
// orthogonality only duplicates converged Ritz values and leaves the extremal
// ones converging to the spectrum's ends); the extremal eigenvalues of the
// tridiagonal matrix T_j come from Sturm-sequence bisection on the host.
// Ritz values lie inside the spectrum, so lambda_min is approached from above
// and lambda_max from below.

#include <algorithm>
#include <cmath>
#include <functional>
#include <random>
#include <vector>

#include "blas_impl.h"
#include "dirac_impl.h"
#include "handles.h"

namespace qed3 {

// number of eigenvalues of the symmetric tridiagonal (a, b) below x
static int sturm_count(const std::vector<double>& a, const std::vector<double>& b, int m, double x) {
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

// k-th smallest eigenvalue (k = 0 .. m-1) of T by bisection on Gershgorin bounds
static double tridiag_eig(const std::vector<double>& a, const std::vector<double>& b, int m, int k) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; i++) {
    const double r = (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i < m - 1 ? std::abs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  for (int it = 0; it < 72 && hi - lo > 1e-16 * std::max(std::abs(lo), std::abs(hi)); it++) {
    const double mid = 0.5 * (lo + hi);
    if (sturm_count(a, b, m, mid) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

int spectral_bounds(qed3_dirac_s* d, double tol, int maxsteps, double* lmin, double* lmax, int* steps_used,
                    cudaStream_t st) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set (call qed3_dirac_set_links)");
  return lanczos_extremal(
      4LL * d->Ns, [&](double* o, const double* v) { return dirac_apply_ref(d, QED3_OP_DDAGD, o, v, st); }, tol,
      maxsteps, lmin, lmax, steps_used, st);
}

int lanczos_extremal(long long nd, const std::function<int(double*, const double*)>& apply, double tol, int maxsteps,
                     double* lmin, double* lmax, int* steps_used, cudaStream_t st) {
  if (!(tol > 0) || maxsteps < 2) return fail(QED3_ERR_ARG, "need tol > 0 and maxsteps >= 2");
  const long long nc = nd / 2;
  double* buf = nullptr;
  if (cudaMalloc(&buf, size_t(nd) * 3 * sizeof(double) + 2048 * sizeof(double)) != cudaSuccess)
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  double *v0 = buf, *v1 = buf + nd, *w = buf + 2 * nd, *part = buf + 3 * nd;
  auto body = [&]() -> int {
    // seeded Gaussian start vector: a component along every eigenvector
    std::vector<double> h(static_cast<size_t>(nd));
    std::mt19937_64 gen(20241203);
    std::normal_distribution<double> nrm;
    for (auto& x : h) x = nrm(gen);
    QED3_CUDA_TRY(cudaMemcpyAsync(v1, h.data(), nd * sizeof(double), cudaMemcpyHostToDevice, st));
    QED3_CUDA_TRY(cudaMemsetAsync(v0, 0, nd * sizeof(double), st));
    double re = 0, im = 0;
    int e = vec_zdot(nc, v1, v1, part, &re, &im, st);
    if (e) return e;
    if ((e = vec_axpby(nd, 1.0 / std::sqrt(re), v1, 0.0, v1, v1, st))) return e;
    std::vector<double> al, be;
    double prev_min = 0, prev_max = 0, beta = 0;
    int j = 0, conv = 0, next_check = 10;
    for (; j < maxsteps; j++) {
      if ((e = apply(w, v1))) return e;
      if (j > 0 && (e = vec_axpby(nd, -beta, v0, 1.0, w, w, st))) return e;
      if ((e = vec_zdot(nc, v1, w, part, &re, &im, st))) return e;
      const double alpha = re;  // real: D^dag D is hermitian
      if ((e = vec_axpby(nd, -alpha, v1, 1.0, w, w, st))) return e;
      if ((e = vec_zdot(nc, w, w, part, &re, &im, st))) return e;
      al.push_back(alpha);
      beta = std::sqrt(std::max(re, 0.0));
      const int m = int(al.size());
      // Ritz values every max(10, m/16) steps: the bisections cost O(m) each
      if (m >= 4 && (m >= next_check || beta == 0.0)) {
        next_check = m + std::max(10, m / 16);
        const double tmin = tridiag_eig(al, be, m, 0), tmax = tridiag_eig(al, be, m, m - 1);
        if (std::abs(tmin - prev_min) <= tol * std::abs(tmin) && std::abs(tmax - prev_max) <= tol * std::abs(tmax))
          conv++;
        else
          conv = 0;
        prev_min = tmin;
        prev_max = tmax;
        if (conv >= 2 || beta == 0.0) {
          j++;
          break;
        }
      }
      be.push_back(beta);
      // v0 <- v1, v1 <- w / beta
      std::swap(v0, v1);
      if ((e = vec_axpby(nd, 1.0 / beta, w, 0.0, w, v1, st))) return e;
    }
    if (conv < 2) {
      const int m = int(al.size());
      prev_min = tridiag_eig(al, be, m, 0);
      prev_max = tridiag_eig(al, be, m, m - 1);
    }
    *lmin = prev_min;
    *lmax = prev_max;
    if (steps_used) *steps_used = j;
    return conv >= 2 ? QED3_OK : QED3_ERR_NOCONV;
  };
  const int rc = body();
  cudaFree(buf);
  return rc;
}

}  // namespace qed3
