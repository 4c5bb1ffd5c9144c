// Zolotarev optimal rational approximation of sign(x) on [k, 1].
//
// Same approximation as the reference's Zolotarev struct
// (src/both_3d/overlap.h:7-134, after A.D. Kennedy, hep-lat/0402038):
//   r(x) = C x (1 + sum_m A_m / (x^2 - k^2/cp_m)),
//   c_m  = -cn^2/sn^2 (2 m K'/n | k'),  cp_m = -cn^2/sn^2 ((2m-1) K'/n | k'),
// with K' = K(k').  The Jacobi functions are evaluated here by the
// arithmetic-geometric-mean method of Abramowitz & Stegun 16.4 (descending
// Landen sequence with backward phase recursion) instead of the reference's
// recursive Gauss transformation, and K' from the same AGM.

#include <cmath>
#include <vector>

#include "qed3_internal.h"

namespace qed3 {
namespace {

// Jacobi sn, cn, dn of argument u and modulus k (A&S 16.4.3); also K(k).
void jacobi(double u, double k, double& sn, double& cn, double& dn, double& K) {
  const int NMAX = 64;
  double a[NMAX + 1], c[NMAX + 1];
  double aa = 1.0, bb = std::sqrt((1.0 - k) * (1.0 + k));
  a[0] = aa;
  c[0] = k;
  int n = 0;
  while (n < NMAX) {
    const double an = 0.5 * (aa + bb), bn = std::sqrt(aa * bb), cn_ = 0.5 * (aa - bb);
    n++;
    a[n] = an;
    c[n] = cn_;
    aa = an;
    bb = bn;
    if (std::abs(cn_) <= 1e-17 * an) break;
  }
  K = M_PI / (2.0 * a[n]);
  double phi = std::ldexp(a[n] * u, n);  // 2^n a_n u
  double phi_next = phi;
  for (int j = n; j >= 1; j--) {
    phi_next = phi;
    phi = 0.5 * (phi + std::asin(c[j] / a[j] * std::sin(phi)));
  }
  sn = std::sin(phi);
  cn = std::cos(phi);
  // dn = cos(phi_0) / cos(phi_1 - phi_0)
  dn = (n >= 1) ? cn / std::cos(phi_next - phi) : 1.0;
}

}  // namespace

int zolotarev_coeffs(double k, int n, ZoloCoeffs& z) {
  if (!(k > 0.0 && k < 1.0) || n < 1) return fail(QED3_ERR_ARG, "Zolotarev needs 0 < k < 1 and order >= 1");
  z = ZoloCoeffs{};
  z.n = n;
  z.k = k;
  z.size = n / 2 + 1;
  const int S = z.size;
  z.c.assign(S, 0.0);
  z.cp.assign(S, 0.0);
  z.A.assign(S, 0.0);
  const double kp = std::sqrt((1.0 - k) * (1.0 + k));
  double sn, cn, dn, Kp;
  jacobi(0.0, kp, sn, cn, dn, Kp);
  double xibar = 1.0;
  for (int m = 1; m < S; m++) {
    double K_;
    jacobi(2.0 * Kp * m / n, kp, sn, cn, dn, K_);
    z.c[m] = -(cn / sn) * (cn / sn);
    jacobi(2.0 * Kp * (m - 0.5) / n, kp, sn, cn, dn, K_);
    z.cp[m] = -(cn / sn) * (cn / sn);
    if (m == 1) xibar = 1.0 / dn;
  }
  double M = 1.0;
  for (int m = 1; m < S; m++) M *= (1.0 - z.c[m]) / (1.0 - z.cp[m]);
  double li = xibar / M;
  for (int m = 1; m < S; m++) li *= (1.0 - z.c[m] * xibar * xibar) / (1.0 - z.cp[m] * xibar * xibar);
  double E = 1.0;
  const double k2 = k * k;
  for (int m = 1; m < S; m++) {
    double num = 1.0, den = 1.0;
    for (int l = 1; l < S; l++) {
      num *= k2 / z.cp[m] - k2 / z.c[l];
      if (l != m) den *= k2 / z.cp[m] - k2 / z.cp[l];
    }
    z.A[m] = num / den;
    E *= z.c[m] / z.cp[m];
  }
  z.M = M;
  z.lambda_inv = li;
  z.E = E;
  z.C = E * 2.0 / (1.0 + li) / (k * M);
  return QED3_OK;
}

}  // namespace qed3
