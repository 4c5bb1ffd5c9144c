// Compiles include/qed3_linop.h inside the reference's own operator and solver
// headers (src/both_3d/gpu_header.h, sparse_matrix.h, matpoly.h; paths passed
// as REF_* macros by tests/test_reference_shim.py) and instantiates the
// reference's MatPoly::solve over Qed3Op, the way a reference driver would:
// the drop-in compiles and links against libqed3.  Running it needs the
// reference headers where the GPU is; the test only builds it.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <vector>

using Idx = std::int32_t;
using Complex = std::complex<double>;
static constexpr int NS = 2;
namespace Comp {
constexpr int N_REFINE = 8;
constexpr int Nt = 1;
constexpr Idx N_SITES = 20 * N_REFINE * N_REFINE;
constexpr Idx Nx = NS * N_SITES;
constexpr Idx N = Nx * Nt;
const double TOL_INNER = 1.0e-15;
const double TOL_OUTER = 1.0e-14;
}  // namespace Comp

#include <cublas_v2.h>
#include <cuComplex.h>
#include <cuda_runtime.h>
using CuC = cuDoubleComplex;
#include REF_GPU_HEADER_H
#include REF_SPARSE_MATRIX_H
#include REF_MATPOLY_H

#include "qed3_linop.h"

// A reference-style propagator solve: MatPoly over {D, D^dag} through the C ABI.
int reference_cg_over_qed3(qed3_dirac* d, CuC* d_x, const CuC* d_b, double tol) {
  Qed3Op M_DW(d, QED3_OP_D), M_DWH(d, QED3_OP_DDAG);
  MatPoly Op;
  Op.push_back(cplx(1.0), {&M_DW, &M_DWH});
  Op.solve<Comp::N>(d_x, d_b, tol, 100000);
  Qed3Solver fast(d, QED3_PREC_F32);  // the same solve by the library's own CG
  fast.solve(d_x, d_b, tol, 100000);
  return 0;
}

int main() {
  qed3_lattice* lat = nullptr;
  qed3_dirac* d = nullptr;
  if (qed3_lattice_create(Comp::N_REFINE, &lat) != QED3_OK) return 1;
  if (qed3_dirac_create(lat, 1.0, 0.1, &d) != QED3_OK) return 1;
  std::printf("shim built: N = %d\n", int(Comp::N));
  (void)reference_cg_over_qed3;
  qed3_dirac_destroy(d);
  qed3_lattice_destroy(lat);
  return 0;
}
