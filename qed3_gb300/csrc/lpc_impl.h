// Learned preconditioner (lpc.cu): handle and host entry points.
//
// The network N(r) = a^2 r + G^dag G r, G = L_LG o ... o L_1, each layer a
// gauge-covariant parallel-transport convolution on the dual lattice:
//   L(h)[c] = sum_c' W0[c,c'] h[c'] + W1[c,c'] Hd(h)[c'] + W2[c,c'] Ho(h)[c']
// Hd / Ho apply the diagonal / off-diagonal part of the Dirac hop block
// H_xy = kappa/2 (-r + gamma_xy) e^{iA} Omega_xy from the in-block neighbours
// (blocks = the persistent solver's per-SM site ranges).  Under
// gamma5-hermiticity Hd is self-adjoint and Ho anti-self-adjoint, so G^dag
// reuses the same tables and N is hermitian positive definite by construction
// -- the property that keeps preconditioned CG's short recurrence valid.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "handles.h"
#include "tc_impl.h"

namespace qed3 {
constexpr int kLpcMaxWords = 7;  // hop words of length <= 2 over {Hd, Ho} (incl. identity)
struct LpcWordCoef {              // collapsed form used inside the solver
  float2 M[kLpcMaxWords][kLpcMaxWords];  // hermitian PSD, row-major M[w][w']
  float a2;
  int nwords;
  int per;                        // sites per block (the block mask)
};
}  // namespace qed3

struct qed3_lpc_s {
  int C = 16, LG = 2, per = 544, Ns = 0;
  qed3_dirac_s* d = nullptr;
  // parameters: per layer 3 x Cout x Cin complex (fp32 master copy), then a
  std::vector<int> cin, cout, woff;  // per layer
  int nparam = 0;                     // complex entries incl. a (stored as (a, 0))
  float2* W = nullptr;                // device [nparam]
  float2* G = nullptr;                // gradient
  float2* m = nullptr;                // Adam moments
  float2* v = nullptr;
  int adam_t = 0;
  // activations for a batch
  int bmax = 0;
  std::vector<float2*> act;  // h0..hLG, g_{LG-1}..g0 (fields [B][Ns][C][2] complex)
  float2 *fa = nullptr, *fb = nullptr, *tmp = nullptr, *gz = nullptr, *az = nullptr, *mid = nullptr;
  double* part = nullptr;
  // training pairs (internal order, fp32 complex two-spinors)
  float2* R = nullptr;
  float2* E = nullptr;
  int npairs = 0, cap_pairs = 0;
  std::vector<qed3::M32*> cfg_H;   // hop blocks (fp32) of D for every operator pairs came from
  std::vector<qed3::M32*> cfg_Hd;  // and of D^dag
  std::vector<int> pair_cfg;       // operator index of each pair
  float2* bR = nullptr;            // batch gather buffers
  float2* bE = nullptr;
  // collapsed form, cached until the weights change
  bool coef_valid = false;
  qed3::LpcWordCoef coef{};
  // 16 -> 16 layers on the tensor cores (bf16 operands, fp32 accumulation)
  bool use_tc = false;
  int sms = 0;
  qed3::TcWork tc;
};

namespace qed3 {
int lpc_create(qed3_dirac_s* d, int channels, int layers, int per, unsigned seed, qed3_lpc_s** out);
void lpc_destroy(qed3_lpc_s* L);
int lpc_forward(qed3_lpc_s* L, int B, const float2* r, float2* z, cudaStream_t st);
int lpc_loss_grad(qed3_lpc_s* L, int B, const float2* r, const float2* e, double* loss, cudaStream_t st);
int lpc_adam(qed3_lpc_s* L, double lr, cudaStream_t st);
int lpc_word_coef(const qed3_lpc_s* L, LpcWordCoef* out);
int lpc_word_coef_cached(qed3_lpc_s* L, LpcWordCoef* out);
int lpc_get_weights(const qed3_lpc_s* L, double* w);
int lpc_set_weights(qed3_lpc_s* L, const double* w);
int lpc_apply_words(qed3_lpc_s* L, int B, const float2* r, float2* z, cudaStream_t st);
int lpc_collect(qed3_lpc_s* L, qed3_dirac_s* d, int nsrc, unsigned seed, const int* snaps, int nsnap, int prec);
int lpc_train(qed3_lpc_s* L, int steps, int batch, double lr, unsigned seed, double* history);
int lpc_set_tensor_cores(qed3_lpc_s* L, int enable);
}  // namespace qed3
