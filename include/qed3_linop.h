/* C++ adaptor of the qed3 C ABI to the reference's operator interface.
 *
 * Include after the reference's sparse_matrix.h (src/both_3d/sparse_matrix.h
 * or src/dual/sparse_matrix.h), which defines LinOp, CuC and CUDA_CHECK; link
 * with -lqed3.  Qed3Op replaces the CSR operator (sparse_matrix.h:12-39) in a
 * MatPoly product chain, so the reference's own MatPoly::solve
 * (src/both_3d/matpoly.h:204-267) runs over this library's stencil apply:
 *
 *     Qed3Op M_DW(d, QED3_OP_D), M_DWH(d, QED3_OP_DDAG);
 *     MatPoly Op;  Op.push_back(cplx(1.0), {&M_DW, &M_DWH});
 *     Op.solve<N>(d_x, d_b, tol, maxiter);
 *
 * Qed3Solver is the drop-in for the same call with this library's persistent
 * CG (qed3_cg_solve: FP64 certificate, optional mixed precision). */
#pragma once

#include <stdexcept>

#include "qed3.h"

struct Qed3Op : public LinOp {
  qed3_dirac* d;
  int op;  // QED3_OP_D, QED3_OP_DDAG, QED3_OP_DDAGD or QED3_OP_DDDAG
  Qed3Op(qed3_dirac* d_, int op_) : d(d_), op(op_) {}
  void operator()(CuC* res, const CuC* v) const override {
    if (qed3_dirac_apply(d, op, reinterpret_cast<double*>(res), reinterpret_cast<const double*>(v), nullptr) !=
        QED3_OK)
      throw std::runtime_error(qed3_last_error_string());
  }
  void Async(CuC* res, const CuC* v, const cudaStream_t s) const override {
    if (qed3_dirac_apply(d, op, reinterpret_cast<double*>(res), reinterpret_cast<const double*>(v), (void*)s) !=
        QED3_OK)
      throw std::runtime_error(qed3_last_error_string());
    CUDA_CHECK(cudaStreamSynchronize(s));  // the reference's Async returns after the product
  }
};

struct Qed3Solver {
  qed3_dirac* d;
  int precision;  // QED3_PREC_F64 / _F32 / _BF16
  explicit Qed3Solver(qed3_dirac* d_, int precision_ = QED3_PREC_F64) : d(d_), precision(precision_) {}
  // MatPoly::solve<N>(d_x, d_b, tol, maxiter) on D^dag D
  void solve(CuC* d_x, const CuC* d_b, double tol, int maxiter) const {
    qed3_solve_params p{tol, maxiter, precision, 0.1, 0.0, 0};
    qed3_solve_report r;
    const int rc = qed3_cg_solve(d, reinterpret_cast<double*>(d_x), reinterpret_cast<const double*>(d_b), &p, &r,
                                 nullptr);
    if (rc != QED3_OK) throw std::runtime_error(qed3_last_error_string());
  }
};
