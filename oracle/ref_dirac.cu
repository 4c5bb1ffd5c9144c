// Builds the reference's own Dirac-operator pipeline from the reference tree,
// in place, into oracle/_ref/libdirac_ref_n<n>_t<Nt>.so (one library per
// refinement and number of time slices: the reference fixes both at compile
// time in namespace Comp).  Test infrastructure only: it pins the oracle's
// restatement and, through the golden fixture it writes, the GPU operator.
//
// What runs is the reference's code, compiled from its headers:
//   S2Simp          src/both_3d/s2n_simp.h:43-402   reads the .dat tables, triangle
//                                                  areas, link lengths, dual areas
//   S2Trivalent     src/both_3d/s2n_dual.h:49-166   dual lattice, link volumes
//   SpinStructureDual, DiracS2Dual
//                   src/both_3d/dirac_dual.h:15-215 omega/alpha tables, the
//                                                  spin-structure check, kappa,
//                                                  gamma, Omega
//   DiracExt        src/both_3d/dirac_ext.h:6-334   coo_structure, coo_format
//   GaugeExt        src/both_3d/gauge_ext.h         link angles, sp/tp (FermionVector
//                   from src/both_3d/valence.h for its declarations)
//   DWDevice        src/both_3d/sparse_dirac.h      COO -> CSR of D and D^dagger
//   matmul          src/both_3d/sparse_matrix.h:257-270  host CSR SpMV
// The tables are read from a directory of .dat files in the reference's
// layout (written by qed3_gb300.dats.write from this project's lattice).
//
// Adaptations, none of which changes the arithmetic of the code above:
//   * VE and MS are small stand-ins for the two Eigen types those headers use
//     (a 3-vector; a 2x2 complex matrix with comma initialisation); Eigen is
//     not installed.  oracle/ref_shim/Eigen/Dense is an empty header.
//   * DWDevice uploads its arrays to the GPU; no GPU exists where this runs,
//     so its CUDA calls are made with a no-op error check and fail
//     harmlessly.  Only its host CSR assembly and permutation are used.
//   * MatPoly::solve (src/both_3d/matpoly.h:204-267) drives device buffers
//     and cuBLAS and cannot run without a GPU.  ref_dirac_run restates its
//     iteration step for step on the host, over the reference's own matmul
//     and CSR arrays, to record the CG iterates.
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef NDEBUG
#error "the reference's assertions are part of the pin: build without NDEBUG"
#endif

using Double = double;
using Idx = std::int32_t;
using Complex = std::complex<double>;
using Link = std::array<Idx, 2>;
using Face = std::vector<Idx>;

// 3-vector stand-in (the members of Eigen::Vector3d that the headers call).
struct VE {
  double c[3] = {0.0, 0.0, 0.0};
  VE() = default;
  VE(double a, double b, double d) : c{a, b, d} {}
  double dot(const VE& o) const { return c[0] * o.c[0] + c[1] * o.c[1] + c[2] * o.c[2]; }
  double norm() const { return std::sqrt(dot(*this)); }
  VE cross(const VE& o) const {
    return VE(c[1] * o.c[2] - c[2] * o.c[1], c[2] * o.c[0] - c[0] * o.c[2], c[0] * o.c[1] - c[1] * o.c[0]);
  }
  VE operator-(const VE& o) const { return VE(c[0] - o.c[0], c[1] - o.c[1], c[2] - o.c[2]); }
  VE operator+(const VE& o) const { return VE(c[0] + o.c[0], c[1] + o.c[1], c[2] + o.c[2]); }
};

// 2x2 complex matrix stand-in (Eigen::Matrix2cd): comma initialisation in
// row order, element access, sums, scalar and matrix products.
struct MS {
  Complex e[4];
  struct Init {
    MS* m;
    int k;
    template <typename T>
    Init& operator,(const T& v) {
      m->e[k++] = Complex(v);
      return *this;
    }
  };
  template <typename T>
  Init operator<<(const T& v) {
    e[0] = Complex(v);
    return Init{this, 1};
  }
  Complex& operator()(int i, int j) { return e[2 * i + j]; }
  const Complex& operator()(int i, int j) const { return e[2 * i + j]; }
};
inline MS operator+(const MS& a, const MS& b) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = a.e[k] + b.e[k];
  return r;
}
inline MS operator-(const MS& a, const MS& b) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = a.e[k] - b.e[k];
  return r;
}
inline MS operator-(const MS& a) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = -a.e[k];
  return r;
}
inline MS operator*(const MS& a, const MS& b) {
  MS r;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) r(i, j) = a(i, 0) * b(0, j) + a(i, 1) * b(1, j);
  return r;
}
inline MS operator*(const Complex& s, const MS& a) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = s * a.e[k];
  return r;
}
inline MS operator*(const MS& a, const Complex& s) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = a.e[k] * s;
  return r;
}
inline MS operator*(double s, const MS& a) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = s * a.e[k];
  return r;
}
inline MS operator*(const MS& a, double s) {
  MS r;
  for (int k = 0; k < 4; k++) r.e[k] = a.e[k] * s;
  return r;
}

static constexpr int NS = 2;
static constexpr int DIM = 2;
static constexpr Complex I = Complex(0.0, 1.0);

namespace Comp {
constexpr bool is_compact = false;
constexpr int NPARALLEL_DUPDATE = 1;
constexpr int NPARALLEL = 1;
constexpr int NSTREAMS = 1;
constexpr int NPARALLEL_GAUGE = 1;
constexpr int NPARALLEL_SORT = 8;
constexpr int N_REFINE = REF_NREF;
constexpr int NS = 2;
constexpr int Nt = REF_NT;
constexpr Idx N_SITES = 20 * N_REFINE * N_REFINE;
constexpr Idx Nx = NS * N_SITES;
constexpr Idx N = Nx * Nt;
const double TOL_INNER = 1.0e-15;
const double TOL_OUTER = 1.0e-14;
}  // namespace Comp

// The directory the reference's table readers prepend to every file name.
std::string dir;

#include REF_S2N_SIMP_H
#include REF_S2N_DUAL_H
#include REF_VALENCE_H  // FermionVector, named by GaugeExt::gauge_trsf
#include REF_GAUGE_EXT_H

#include <cublas_v2.h>
#include <cuComplex.h>
#include <cuda_runtime.h>
using CuC = cuDoubleComplex;
#include REF_GPU_HEADER_H
#include REF_SPARSE_MATRIX_H
#include REF_DIRAC_BASE_H
#include REF_DIRAC_DUAL_H
#include REF_DIRAC_EXT_H
#undef CUDA_CHECK
#define CUDA_CHECK(err) ((void)(err))
#include REF_SPARSE_DIRAC_H

namespace {
using Dirac = DiracExt<S2Trivalent, DiracS2Dual>;
using Gauge = GaugeExt<S2Trivalent, Comp::Nt, false>;
constexpr Idx N = Comp::N;

// Silences the readers' progress lines while the reference objects are built.
struct Quiet {
  std::stringstream sink;
  std::streambuf *o, *l;
  Quiet() : o(std::cout.rdbuf(sink.rdbuf())), l(std::clog.rdbuf(sink.rdbuf())) {}
  ~Quiet() {
    std::cout.rdbuf(o);
    std::clog.rdbuf(l);
  }
};

std::vector<CuC> to_cuc(const std::vector<Complex>& v) {
  std::vector<CuC> out(v.size());
  for (size_t i = 0; i < v.size(); i++) out[i] = make_cuDoubleComplex(v[i].real(), v[i].imag());
  return out;
}

CuC zdotc(const std::vector<CuC>& x, const std::vector<CuC>& y) {
  double re = 0.0, im = 0.0;
  for (Idx i = 0; i < N; i++) {
    re += x[i].x * y[i].x + x[i].y * y[i].y;
    im += x[i].x * y[i].y - x[i].y * y[i].x;
  }
  return make_cuDoubleComplex(re, im);
}
}  // namespace

extern "C" int ref_dirac_config(int* n_refine, int* nt, int* n) {
  *n_refine = Comp::N_REFINE;
  *nt = Comp::Nt;
  *n = N;
  return 0;
}

// Builds the operator from the tables in dat_dir with link angles A
// ([Nt][n_links] spatial, then [Nt][n_sites] temporal, GaugeExt's layout) and
// applies it to v: Dv = D v, DHv = D^dag v, DHDv = D^dag D v (complex
// interleaved, index Nx s + 2 x + spin).  csr_* receive D's CSR arrays
// (rows [N+1], cols and values [len]) and kappa the per-link kappa, each when
// non-null.  The CG on D^dag D x = v (MatPoly::solve, x0 = 0, stop on the
// recursive |r|^2 < tol^2 |b|^2) records x after the iteration counts in
// iters_at[0..n_at) into x_at ([n_at][N] complex) and the converged x into
// x_final; returns the CG's iteration count, or -1 on a bad argument.
extern "C" int ref_dirac_run(const char* dat_dir, double r, double M5, double at, const double* A,
                             const double* v, double* Dv, double* DHv, double* DHDv, int* csr_rows, int* csr_cols,
                             double* csr_val, double* kappa, double tol, int maxiter, int n_at, const int* iters_at,
                             double* x_at, double* x_final) {
  dir = std::string(dat_dir) + "/";
  Quiet* q = new Quiet;
  S2Trivalent lattice(Comp::N_REFINE);
  Dirac D(lattice, 0.0, r, M5, at);
  // DWDevice's destructor would free device buffers that were never made;
  // it is deliberately not destroyed (test infrastructure, small).
  auto* dev = new DWDevice<Dirac>(D);
  Gauge U(lattice);
  for (int s = 0; s < Comp::Nt; s++) {
    for (Idx l = 0; l < lattice.n_links; l++) U.sp(s, l) = A[size_t(s) * lattice.n_links + l];
    for (Idx x = 0; x < lattice.n_sites; x++)
      U.tp(s, x) = A[size_t(Comp::Nt) * lattice.n_links + size_t(s) * lattice.n_sites + x];
  }
  dev->update(U);
  delete q;
  if (lattice.n_sites != Comp::N_SITES) return -1;

  const std::vector<CuC> val = to_cuc(dev->v_csr), valH = to_cuc(dev->v_csrH);
  const std::vector<Idx>&rows = dev->rows_csr, &cols = dev->cols_csr;
  const std::vector<Idx>&rowsT = dev->rows_csrT, &colsT = dev->cols_csrT;
  if (csr_rows) std::memcpy(csr_rows, rows.data(), sizeof(Idx) * rows.size());
  if (csr_cols) std::memcpy(csr_cols, cols.data(), sizeof(Idx) * cols.size());
  if (csr_val) std::memcpy(csr_val, val.data(), sizeof(CuC) * val.size());
  if (kappa) std::memcpy(kappa, D.bd.kappa.data(), sizeof(double) * D.bd.kappa.size());

  auto mD = [&](CuC* o, const CuC* in) { matmul<N>(o, in, val, cols, rows); };
  auto mDH = [&](CuC* o, const CuC* in) { matmul<N>(o, in, valH, colsT, rowsT); };
  std::vector<CuC> vin(N), t(N);
  std::memcpy(vin.data(), v, sizeof(CuC) * N);
  mD(reinterpret_cast<CuC*>(Dv), vin.data());
  mDH(reinterpret_cast<CuC*>(DHv), vin.data());
  mD(t.data(), vin.data());
  mDH(reinterpret_cast<CuC*>(DHDv), t.data());

  // MatPoly::solve<N>(d_x, d_b, tol, maxiter), step for step on the host
  std::vector<CuC> x(N, cplx(0.0)), q2(N, cplx(0.0)), rr(vin), p(vin);
  double mu = real(zdotc(rr, rr));
  double mu_old = mu;
  const double b_norm_sq = real(zdotc(rr, rr));
  const double mu_crit = tol * tol * b_norm_sq;
  int done = 0, next = 0;
  if (!(mu < mu_crit)) {
    int k = 0;
    for (; k < maxiter; ++k) {
      mD(t.data(), p.data());  // on_gpu over {D, D^dag}: D first, then D^dag
      mDH(q2.data(), t.data());
      const CuC gam = zdotc(p, q2);
      const CuC al = cplx(mu) / gam;
      for (Idx i = 0; i < N; i++) x[i] = al * p[i] + x[i];
      for (Idx i = 0; i < N; i++) rr[i] = (-al) * q2[i] + rr[i];
      mu = real(zdotc(rr, rr));
      while (next < n_at && iters_at[next] == k + 1) {
        std::memcpy(x_at + size_t(next) * 2 * N, x.data(), sizeof(CuC) * N);
        next++;
      }
      if (mu < mu_crit || std::isnan(mu)) break;
      const CuC bet = cplx(mu / mu_old);
      mu_old = mu;
      for (Idx i = 0; i < N; i++) p[i] = bet * p[i] + rr[i];
    }
    done = k < maxiter ? k + 1 : k;
  }
  std::memcpy(x_final, x.data(), sizeof(CuC) * N);
  return done;
}
