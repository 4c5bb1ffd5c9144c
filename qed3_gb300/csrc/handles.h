// Handle structures behind the opaque C types of include/qed3.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "qed3_internal.h"

namespace qed3 {
struct S64;
struct M64;
struct M32;
struct GridBar;
struct GridBar2;

#define QED3_CUDA_TRY(call)                                                                        \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return ::qed3::fail(QED3_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

// Device copies of the lattice tables, SoA over the three hop slots, in the
// space-filling-curve (internal) order.
struct DeviceLattice {
  int Ns = 0, Nl = 0, Nf = 0, face_total = 0;
  int32_t* nbr = nullptr;       // [3][Ns] internal neighbour ids
  int32_t* nbr_ref = nullptr;   // [3][Ns] reference ids of the neighbours
  int32_t* perm = nullptr;      // [Ns] internal -> reference
  int32_t* iperm = nullptr;     // [Ns] reference -> internal
  int32_t* hop_link = nullptr;  // [3][Ns]
  int8_t* hop_sign = nullptr;   // [3][Ns]
  int32_t* face_off = nullptr;  // [Nf+1]
  int32_t* face_link = nullptr; // [face_total]
  int8_t* face_sign = nullptr;  // [face_total]
  double* face_weight = nullptr;// [Nf] mean_vol / vols
  int32_t* link_x = nullptr;    // [Nl] internal id of links[l][0]
  int32_t* link_y = nullptr;    // [Nl] internal id of links[l][1]
  int8_t* link_kx = nullptr;    // [Nl] slot of y in x's hops
  int8_t* link_ky = nullptr;    // [Nl] slot of x in y's hops
};

struct SolverWork {
  size_t ns = 0;
  // FP64 internal fields
  S64 *b = nullptr, *xhi = nullptr, *xhi2 = nullptr, *rhi = nullptr, *t64 = nullptr;
  // FP32 fields (also used as FP64 scratch when the solve is plain FP64)
  void *r = nullptr, *p = nullptr, *t = nullptr, *xlo = nullptr, *rg = nullptr, *tg = nullptr;
  double* partials = nullptr;  // [2][maxblocks][4]
  GridBar* bar = nullptr;
  GridBar2* bar2 = nullptr;
  double* scal = nullptr;      // device scalars for the report
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

// Device state of the gauge side (allocated on first use).
struct GaugeDev {
  bool ready = false;
  int32_t* link_face = nullptr;  // [Nl][2] the two dual faces of each link
  int8_t* link_fsign = nullptr;  // [Nl][2] orientation of the link in each
  double *th0 = nullptr, *th1 = nullptr, *pi = nullptr, *pi0 = nullptr, *F = nullptr, *A0 = nullptr;
  double* part = nullptr;
};

}  // namespace qed3

struct qed3_lattice_s {
  qed3::HostLattice host;
  qed3::DeviceLattice dev;
  qed3::GaugeDev gauge;
  int device = 0;
};

struct qed3_dirac_s {
  qed3_lattice_s* lat = nullptr;
  double r = 1.0, M5 = 0.0;
  int Ns = 0;
  std::vector<double> kappa;     // [Nl]
  qed3::M64* G = nullptr;        // [3][Ns] geometric part of H_xy (no U(1) phase)
  qed3::M64* Gd = nullptr;       // [3][Ns] geometric part of (H_yx)^dagger
  qed3::M64* H = nullptr;        // [3][Ns] hop blocks of D
  qed3::M64* Hd = nullptr;       // [3][Ns] hop blocks of D^dagger
  qed3::M32* H32 = nullptr;
  qed3::M32* Hd32 = nullptr;
  double* diag = nullptr;        // [Ns]
  float* diag32 = nullptr;       // [Ns]
  double* A_dev = nullptr;       // [Nl] staging for host link angles
  qed3::S64* tmp_in = nullptr;   // [Ns] scratch for reference-order calls
  qed3::S64* tmp_out = nullptr;
  qed3::S64* tmp_mid = nullptr;
  bool coeffs_set = false;
  qed3::SolverWork work;
  qed3_solve_report last{};
  int sm_count = 0;
};
