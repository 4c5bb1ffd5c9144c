// Builds the reference's own Zolotarev coefficients (src/both_3d/overlap.h:7-134)
// from the reference tree, in place, into oracle/_ref/libzolo_ref.so.  Test
// infrastructure only: it pins the oracle's Zolotarev restatement.  The
// stubs below only satisfy names that the (never instantiated) Overlap
// template in the same header refers to; nothing here is copied from the
// reference.
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <initializer_list>
#include <vector>
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cublas_v2.h>

using Idx = std::int32_t;
using Complex = std::complex<double>;
using CuC = cuDoubleComplex;
namespace Comp {
constexpr Idx N = 2;
constexpr int NSTREAMS = 1;
const double TOL_INNER = 1e-9;
const double TOL_OUTER = 1e-8;
}  // namespace Comp
#define CUDA_CHECK(x) (void)(x)
#define CUBLAS_CHECK(x) (void)(x)
#define CD (sizeof(cuDoubleComplex))
#define H2D (cudaMemcpyHostToDevice)
#define D2D (cudaMemcpyDeviceToDevice)
#define NBlocks 1
#define NThreadsPerBlock 1
inline CuC cplx(double c) { return make_cuDoubleComplex(c, 0.0); }
struct LinOp {};
struct CSR : LinOp {};
template <class W> struct DWDevice {
  explicit DWDevice(const W&) {}
  template <class G> void update(const G&) {}
  void associateCSR(CSR&, bool) {}
};
struct MatPoly {
  MatPoly(cublasHandle_t, cudaStream_t) {}
  void push_back(CuC, std::initializer_list<const LinOp*> = {}) {}
  template <Idx N> void solveAsync(CuC*, const CuC*, double = 0, int = 0) const {}
  template <Idx N> void on_gpuAsync(CuC*, const CuC*) const {}
  template <Idx N> void dotAsync(CuC*, const CuC*, const CuC*) const {}
  template <Idx N> void dot2selfAsync(double*, const CuC*, double = 0) const {}
  template <Idx N> void ZdscalAsync(double, CuC*) const {}
};
template <class T, class T2, Idx N>
__global__ void Taxpy_gen(T*, T2, T*, const T*) {}
inline int omp_get_thread_num() { return 0; }
inline double real(CuC c) { return cuCreal(c); }
struct COO {
  std::vector<int> en;
  void do_it() {}
  void Async(CuC*, const CuC*, cudaStream_t) const {}
  void operator()(CuC*, const CuC*) const {}
};

#include REF_OVERLAP_H

extern "C" int ref_zolotarev(double k, int n, double* c, double* cp, double* A, double* scal) {
  Zolotarev z(k, n);
  for (int m = 0; m < z.size; m++) {
    c[m] = z.c[m];
    cp[m] = z.cp[m];
    A[m] = z.A[m];
  }
  scal[0] = z.M;
  scal[1] = z.lambda_inv;
  scal[2] = z.E;
  scal[3] = z.C;
  return z.size;
}
