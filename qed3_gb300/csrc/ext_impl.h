// S^2 x S^1 operator (ext.cu).
#pragma once

#include <cuda_runtime.h>

#include <functional>

#include "handles.h"

struct qed3_dirac_ext_s {
  qed3_dirac_s* d2 = nullptr;  // the dual-lattice operator: geometry blocks, kappa, diagonal
  int Nt = 1;
  double at = 1.0, r = 1.0;
  qed3::M64* H3 = nullptr;     // [Nt][3][Ns] spatial blocks of D per slice (reference site order)
  qed3::M64* Hd3 = nullptr;    // [Nt][3][Ns] the same for D^dagger
  double* kt = nullptr;        // [Ns] kappa_t (reference order)
  double* diag3 = nullptr;     // [Ns] (reference order)
  double2* Pt = nullptr;       // [Nt][Ns] temporal phases e^{i A_t} (reference order)
  int32_t* nbrR = nullptr;     // [3][Ns] reference ids of the neighbours of reference site x
  // FP32 copies for the mixed-precision CG (allocated at its first use)
  qed3::M32* H3f = nullptr;
  qed3::M32* Hd3f = nullptr;
  float2* Ptf = nullptr;
  float* diag3f = nullptr;
  float* ktf = nullptr;
  float4* fwork = nullptr;     // [5][Nt][Ns] FP32 CG vectors
  bool f32_current = false;    // FP32 copies match the current links
  qed3::S64* tmp = nullptr;    // [Nt][Ns]
  void* work = nullptr;        // CG vectors
  bool links_set = false;
};

struct qed3_overlap_ext_s;

namespace qed3 {
// A chunk of solver iterations (kernel launches only) captured once per solve
// as a CUDA graph on a private stream and replayed on the caller's stream: one
// launch per chunk instead of seven per iteration.  If the capture fails the
// solver launches the kernels directly.
// Two timing events destroyed on every exit path of the solve that owns them.
struct EventPair {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~EventPair() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  cudaError_t create() {
    cudaError_t e = cudaEventCreate(&e0);
    return e != cudaSuccess ? e : cudaEventCreate(&e1);
  }
};

struct IterGraph {
  cudaGraphExec_t exec = nullptr;
  ~IterGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  bool build(int reps, const std::function<int(cudaStream_t)>& iter) {
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    int rc = 0;
    for (int k = 0; ok && k < reps && !rc; k++) rc = iter(cs);
    cudaGraph_t g = nullptr;
    if (ok) ok = cudaStreamEndCapture(cs, &g) == cudaSuccess && rc == 0 && g != nullptr;
    if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (!ok) {
      exec = nullptr;
      cudaGetLastError();
    }
    return ok;
  }
};

int ext_init(qed3_dirac_ext_s* e);
void ext_free(qed3_dirac_ext_s* e);
int ext_set_links(qed3_dirac_ext_s* e, const double* A, cudaStream_t st);
int ext_apply(qed3_dirac_ext_s* e, int op, double* out, const double* in, cudaStream_t st);
int ext_fermion_force(qed3_dirac_ext_s* e, const double* eta, double* F, cudaStream_t st);
int ext_force_bilinear(qed3_dirac_ext_s* e, const double* chi, const double* eta, double c, int acc, double* F,
                       cudaStream_t st);
int ext_propagator(qed3_dirac_ext_s* e, int s, int ix, int a, int dagger, double* sink, const qed3_solve_params* prm,
                   qed3_solve_report* rep, cudaStream_t st);
int ext_overlap_create(qed3_dirac_ext_s* e, int order, qed3_overlap_ext_s** out);
void ext_overlap_destroy(qed3_overlap_ext_s* ov);
int ext_overlap_update(qed3_overlap_ext_s* ov, double lmin, double lmax, double tol, double margin, cudaStream_t st);
int ext_overlap_apply(qed3_overlap_ext_s* ov, int op, double* out, const double* in, double tol, int* iters,
                      cudaStream_t st);
int ext_overlap_solve(qed3_overlap_ext_s* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                      int prop, qed3_solve_report* rep, cudaStream_t st);
void ext_overlap_info(const qed3_overlap_ext_s* ov, double* lmin, double* lmax, double* k, double* delta);
qed3_dirac_ext_s* ext_overlap_operator(qed3_overlap_ext_s* ov);
int ext_overlap_force(qed3_overlap_ext_s* ov, const double* eta, double* F, double tol, int* iters, cudaStream_t st);
// ov != NULL: overlap fermions (bounds fixed to lmin_fix, lmax_fix, or recomputed at every update when 0)
int hmc_ext(qed3_dirac_ext_s* e, qed3_rng_s* rng, double* A, double at, double gsq, double tmax, int nsteps,
            int nsteps_inner, int npf, int integrator, double tol, int prec, int no_reject, int* accepted,
            double* dH_out, int* cg_iters, cudaStream_t st, qed3_overlap_ext_s* ov = nullptr, double tol_inner = 1e-12,
            double lmin_fix = 0.0, double lmax_fix = 0.0);
// FP64 CG on op + shift, op = QED3_OP_DDAGD (default) or QED3_OP_DDDAG
int ext_cg(qed3_dirac_ext_s* e, double* x, const double* b, const qed3_solve_params* prm, qed3_solve_report* rep,
           cudaStream_t st, int op = QED3_OP_DDAGD);
}  // namespace qed3
