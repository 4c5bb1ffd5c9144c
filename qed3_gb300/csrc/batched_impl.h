// Batched persistent solver: device descriptors and host entry points.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "handles.h"

namespace qed3 {

constexpr int kMaxTile = 8;  // right-hand sides per system (compile-time tile)

struct BatchSys {
  int Ns, nrhs, blk0, blk1;
  int ch0, ch1;  // site tiles of this system in the dynamic schedule's tile list
  const int* nbr;
  const M64* H;
  const M64* Hd;
  const double* diag;
  const M32* H32;
  const M32* Hd32;
  const float* diag32;
  double shift[kMaxTile];
  const S64* b;
  S64* xhi;
  S64* xhi2;
  S64* t64;
  void* r;
  void* p;
  void* t;
  void* xlo;
  void* rh;      // bf16 copies of r and t for the neighbour gathers (bf16 mode)
  void* th;
  double* scal;  // [nrhs][6]: mu_true, bnorm2, iters, reliable updates, status, x buffer
  double* bnorm; // [nrhs]: |b| of each right-hand side (the kernel solves for b / |b|)
};

struct BatchArgs {
  const BatchSys* sys;
  const int* sys_of_block;
  int nsys;
  double* partials;
  GridBar* bar;
  int* status;
  double tol2, delta2;
  int maxiter;
  long long spin_limit;
};

// Dynamic schedule: the CG state of each system lives in device memory and
// warps take work items (a step of one system's site tile) in order from one
// counter; the warp that completes a system's last tile of a step reduces its
// tile partials, advances its state and releases the system's next step.
template <int R>
struct DynState {
  int state, iter, nru, xsel;
  int active[R], status[R], it_done[R];
  double mu[R], mu_max[R], beta[R], bnorm2[R], alpha[R], mu_true[R];
  double2 a_r[R];
};

struct DynArgs {
  const BatchSys* sys;
  int nsys;
  const int* sys_of_tile;
  int ntiles;
  int spt;        // sites per thread in a tile (a tile is threads x spt consecutive sites)
  void* state;              // DynState<R>[nsys]
  int* sys_cnt;              // [nsys] tiles of the current step done
  int* epoch;                // [nsys] steps completed
  unsigned long long* work;  // next work item (step * ntiles + tile)
  int* ndone;                // systems finished
  double* part;   // [ntiles][3 R]
  GridBar* bar;
  int* status;
  double tol2, delta2;
  int maxiter;
  long long spin_limit;
};

int batch_occupancy(int prec, int R, int threads, int* per_sm);
int batch_dyn_occupancy(int prec, int R, int threads, int* per_sm);
int batch_dyn_launch(int prec, int R, DynArgs& args, int grid, int threads, cudaStream_t st);
int batch_launch(int prec, int R, BatchArgs& args, int grid, int threads, cudaStream_t st);
int batch_import(const BatchSys& s, const qed3_dirac_s* d, const double* b_ref, int R, bool bcast, cudaStream_t st);
int batch_export(const BatchSys& s, const qed3_dirac_s* d, double* x_ref, int R, cudaStream_t st);

}  // namespace qed3

// A batch: user systems split into internal systems of at most R right-hand
// sides, with their workspaces and the block partition of the launch.
struct qed3_batch_s {
  int prec = 0, R = 1, threads = 256, grid = 0;
  int sched = 0;                      // QED3_BATCH_STATIC (fixed block split) or QED3_BATCH_DYNAMIC (tiles per step)
  long long cap = 0;                  // co-resident blocks of the kernel (the partials' size)
  int ntiles = 0;                     // dynamic schedule: site tiles over all systems
  int spt = 1;                        // dynamic schedule: sites per thread in a tile
  int* d_sys_of_tile = nullptr;
  void* d_dyn = nullptr;              // DynState per system
  int* d_counters = nullptr;
  double* d_tile_part = nullptr;
  std::vector<qed3_dirac_s*> user_ops;
  std::vector<int> user_nrhs;
  // internal systems
  std::vector<int> owner, first_rhs;  // user system and its first rhs
  std::vector<qed3::BatchSys> sys;
  std::vector<double> work;           // expected iterations per right-hand side of each system
  std::vector<int> sob;               // block -> system (host copy of d_sys_of_block)
  std::vector<double> last_scal;      // per-right-hand-side scalars of the last reported launch
  qed3::BatchSys* d_sys = nullptr;
  int* d_sys_of_block = nullptr;
  double* partials = nullptr;
  qed3::GridBar* bar = nullptr;
  int* d_status = nullptr;
  double* d_scal = nullptr;
  std::vector<void*> buffers;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool sys_uploaded = false;  // d_sys holds the current descriptors and shifts
  bool timing = false;        // record e0/e1 around the launch (synchronous solves only)
};

namespace qed3 {
int batch_create(int nsys, qed3_dirac_s* const* ops, const int* nrhs, int prec, int rhs_tile, int threads,
                 qed3_batch_s** out, int sched = 0);
void batch_destroy(qed3_batch_s* bt);
int batch_solve(qed3_batch_s* bt, double* const* x, const double* const* b, const double* const* shifts,
                const qed3_solve_params* prm, qed3_solve_report* reports, float* ms_out, cudaStream_t st);
int batch_set_shifts(qed3_batch_s* bt, const double* const* shifts, double shift, cudaStream_t st);
int batch_launch_all(qed3_batch_s* bt, double* const* x, const double* const* b, const qed3_solve_params* prm,
                     cudaStream_t st);
int batch_reports(qed3_batch_s* bt, qed3_solve_report* reports, float ms, cudaStream_t st);
struct BatchTrial {
  int R, threads, sched;
  float ms;
};
int batch_autotune(qed3_batch_s* proto, int* best_R, int* best_threads, int* best_sched, std::vector<BatchTrial>* log);
}  // namespace qed3
