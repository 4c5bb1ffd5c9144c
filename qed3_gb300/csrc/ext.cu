// The S^2 x S^1 operator: Nt time slices of the dual lattice, DiracExt
// (src/both_3d/dirac_ext.h:6-334).  Per time slice s the spatial hops are the
// dual-lattice blocks with that slice's link angles,
//     0.5 kappa_l (-r + gamma(x,y)) e^{i A_s(x,y)} Omega(x,y)        (:135-150),
// the temporal hops between (x, s) and (x, s +- 1) are spin-diagonal,
//     D[(x,s+1),(x,s)] = 0.5 sP kappa_t[x] (-r - sigma3) e^{-i A_t(s,x)},
//     D[(x,s-1),(x,s)] = 0.5 sM kappa_t[x] (-r + sigma3) e^{+i A_t(s-1,x)}
// (:156-184) with the antiperiodic signs sP = -1 at s = Nt-1, sM = -1 at s = 0,
// and the diagonal is M5 + sum_l r kappa_l / 2 + r kappa_t[x] (:188-205) with
// kappa_t[x] = (area of the triangle of x) / mean_ell / at, zero at Nt = 1
// (:297-305).  Vectors are the reference's: index Nx s + 2 x + spin, Nx = 2 Ns.
// Link angles: A[Nt][Nl] spatial then A[Nt][Ns] temporal (GaugeExt's layout).
//
// Spatial blocks per slice and the temporal phases e^{i A_t} are formed once
// per link update (GB300's FP64 pipe is narrow: no sincos in the apply); the
// apply is one kernel per operator, a thread per (slice, site) in the
// reference's site order, so the spinor, block and phase streams are
// coalesced and only the three spatial neighbour reads gather.  CG on
// D^dag D is the reference's MatPoly::solve recurrence in FP64 with device BLAS.

#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "blas_impl.h"
#include "device.cuh"
#include "dirac_impl.h"
#include "ext_impl.h"
#include "handles.h"

namespace qed3 {

static inline int nblk(long long n, int t = 256) { return int((n + t - 1) / t); }

// per-slice spatial blocks in reference site order: H3[s][k][x] = e^{i sgn A_s[l]} G[k][i(x)],
// Hd3 likewise; then the temporal phases Pt[s][x] = e^{i A_t(s, x)}
__global__ void k_ext_set_links(int Ns, int Nl, int Nt, const int32_t* __restrict__ iperm,
                                const int32_t* __restrict__ hop_link, const int8_t* __restrict__ hop_sign,
                                const double* __restrict__ A, const M64* __restrict__ G, const M64* __restrict__ Gd,
                                M64* __restrict__ H3, M64* __restrict__ Hd3, double2* __restrict__ Pt) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nh = 3LL * Ns * Nt;
  if (idx >= nh) {
    const long long t = idx - nh;
    if (t < (long long)Ns * Nt) {
      double sn, cs;
      sincos(A[size_t(Nt) * Nl + t], &sn, &cs);
      Pt[t] = make_double2(cs, sn);
    }
    return;
  }
  const int s = int(idx / (3LL * Ns));
  const int kx = int(idx % (3LL * Ns));
  const int k = kx / Ns, x = kx % Ns;
  const int q = k * Ns + iperm[x];
  const double a = double(hop_sign[q]) * A[size_t(s) * Nl + hop_link[q]];
  double sn, cs;
  sincos(a, &sn, &cs);
  const double2 ph = make_double2(cs, sn);
  const M64 g = G[q], gd = Gd[q];
  H3[idx] = M64{cmul(ph, g.h00), cmul(ph, g.h01), cmul(ph, g.h10), cmul(ph, g.h11)};
  Hd3[idx] = M64{cmul(ph, gd.h00), cmul(ph, gd.h01), cmul(ph, gd.h10), cmul(ph, gd.h11)};
}

// out = op(D) in for op = D (adj = 0) or D^dag (adj = 1), reference order;
// thread (s, x) for reference site x
__global__ void k_ext_apply(int Ns, int Nt, int adj, const int32_t* __restrict__ nbrR,
                            const M64* __restrict__ H3, const double* __restrict__ diag3,
                            const double* __restrict__ kt, const double2* __restrict__ Pt, double r,
                            const S64* __restrict__ in, S64* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Ns * Nt) return;
  const int s = int(idx / Ns), x = int(idx % Ns);
  const S64* vs = in + size_t(s) * Ns;
  const Sp64 self = ld64(vs, x);
  const double dg = diag3[x];
  Sp64 o{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const M64 m = H3[(size_t(s) * 3 + k) * Ns + x];
    const Sp64 b = ld64(vs, nbrR[size_t(k) * Ns + x]);
    o.s0 = cfma(m.h00, b.s0, o.s0);
    o.s0 = cfma(m.h01, b.s1, o.s0);
    o.s1 = cfma(m.h10, b.s0, o.s1);
    o.s1 = cfma(m.h11, b.s1, o.s1);
  }
  if (Nt > 1) {
    const double kh = 0.5 * kt[x];
    const int sp = (s + 1) % Nt, sm = (s + Nt - 1) % Nt;
    const Sp64 up = ld64(in + size_t(sp) * Ns, x), dn = ld64(in + size_t(sm) * Ns, x);
    // spin-diagonal coefficients (upper, lower) and phases of the two hops
    double cu0, cu1, cd0, cd1;
    if (!adj) {
      // from (x, s+1): tmpM(s+1) = 0.5 sM(s+1) kt (-r + sigma3) e^{+i A_t(s,x)}
      const double sgn_u = (sp == 0) ? -1.0 : 1.0;
      cu0 = sgn_u * kh * (-r + 1.0);
      cu1 = sgn_u * kh * (-r - 1.0);
      // from (x, s-1): tmpP(s-1) = 0.5 sP(s-1) kt (-r - sigma3) e^{-i A_t(s-1,x)}
      const double sgn_d = (sm == Nt - 1) ? -1.0 : 1.0;
      cd0 = sgn_d * kh * (-r - 1.0);
      cd1 = sgn_d * kh * (-r + 1.0);
    } else {
      // conj(D[(x,s+1),(x,s)]) = conj(tmpP(s)): sP(s) kt/2 (-r - sigma3) e^{+i A_t(s,x)}
      const double sgn_u = (s == Nt - 1) ? -1.0 : 1.0;
      cu0 = sgn_u * kh * (-r - 1.0);
      cu1 = sgn_u * kh * (-r + 1.0);
      // conj(D[(x,s-1),(x,s)]) = conj(tmpM(s)): sM(s) kt/2 (-r + sigma3) e^{-i A_t(s-1,x)}
      const double sgn_d = (s == 0) ? -1.0 : 1.0;
      cd0 = sgn_d * kh * (-r + 1.0);
      cd1 = sgn_d * kh * (-r - 1.0);
    }
    // both cases: up hop e^{+i A_t(s,x)}, down hop e^{-i A_t(s-1,x)}
    const double2 pu = Pt[size_t(s) * Ns + x], pdc = Pt[size_t(sm) * Ns + x];
    const double2 pd = make_double2(pdc.x, -pdc.y);
    o.s0 = cadd(o.s0, cadd(cscale(cu0, cmul(pu, up.s0)), cscale(cd0, cmul(pd, dn.s0))));
    o.s1 = cadd(o.s1, cadd(cscale(cu1, cmul(pu, up.s1)), cscale(cd1, cmul(pd, dn.s1))));
  }
  st64(out + size_t(s) * Ns, x, o);
}

// Fermion force F = -2 Re <D eta, dD/dA eta> for every link (DiracExt::
// d_coo_format, src/both_3d/dirac_ext.h:234-320); eta, D eta in reference order.
// Spatial link l = (x -> y) of slice s: i H_xy(s) at (x, y) and -i H_yx(s) at (y, x).
__global__ void k_ext_force_sp(int Ns, int Nl, int Nt, const int32_t* __restrict__ lx,
                               const int32_t* __restrict__ ly, const int8_t* __restrict__ kx,
                               const int8_t* __restrict__ ky, const int32_t* __restrict__ perm,
                               const M64* __restrict__ H3, const S64* __restrict__ eta, const S64* __restrict__ deta,
                               double c, int acc, double* __restrict__ F) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Nl * Nt) return;
  const int s = int(idx / Nl), l = int(idx % Nl);
  const int xr = perm[lx[l]], yr = perm[ly[l]];
  const M64 hxy = H3[(size_t(s) * 3 + kx[l]) * Ns + xr], hyx = H3[(size_t(s) * 3 + ky[l]) * Ns + yr];
  const S64* es = eta + size_t(s) * Ns;
  const S64* ds = deta + size_t(s) * Ns;
  const Sp64 ex = ld64(es, xr), ey = ld64(es, yr), dx = ld64(ds, xr), dy = ld64(ds, yr);
  const double2 u0 = cfma(hxy.h01, ey.s1, cmul(hxy.h00, ey.s0));
  const double2 u1 = cfma(hxy.h11, ey.s1, cmul(hxy.h10, ey.s0));
  const double2 v0 = cfma(hyx.h01, ex.s1, cmul(hyx.h00, ex.s0));
  const double2 v1 = cfma(hyx.h11, ex.s1, cmul(hyx.h10, ex.s0));
  // Re[conj(a) (i b)] = a.y b.x - a.x b.y
  auto re_ci = [](double2 a, double2 b) { return a.y * b.x - a.x * b.y; };
  const double f = -2.0 * (re_ci(dx.s0, u0) + re_ci(dx.s1, u1) - re_ci(dy.s0, v0) - re_ci(dy.s1, v1));
  F[idx] = acc ? F[idx] + c * f : c * f;
}

// Temporal link (s, x) from (x, s) to (x, s+1): D[(x,s+1),(x,s)] = tmpP(s) ~ e^{-iA}
// and D[(x,s),(x,s+1)] = tmpM(s+1) ~ e^{+iA}, both with the sign -1 at s = Nt-1:
//   F = -2 Re[ (D eta)_{s+1}^dag (-i tmpP eta_s) + (D eta)_s^dag (i tmpM eta_{s+1}) ]
__global__ void k_ext_force_tp(int Ns, int Nl, int Nt, const double* __restrict__ kt,
                               const double2* __restrict__ Pt, double r, const S64* __restrict__ eta,
                               const S64* __restrict__ deta, double c, int acc, double* __restrict__ F) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Ns * Nt) return;
  const int s = int(idx / Ns), x = int(idx % Ns);
  const int s1 = (s + 1) % Nt;
  const double sg = (s == Nt - 1) ? -1.0 : 1.0;
  const double kh = 0.5 * kt[x] * sg;
  const double cs = Pt[idx].x, sn = Pt[idx].y;
  const Sp64 e0 = ld64(eta + size_t(s) * Ns, x), e1 = ld64(eta + size_t(s1) * Ns, x);
  const Sp64 d0 = ld64(deta + size_t(s) * Ns, x), d1 = ld64(deta + size_t(s1) * Ns, x);
  // tmpP eta_s: spin-diagonal (-r-1, -r+1) kh e^{-iA};  tmpM eta_{s+1}: (-r+1, -r-1) kh e^{+iA}
  const double2 pm = make_double2(cs, -sn), pp = make_double2(cs, sn);
  const double2 a0 = cscale(kh * (-r - 1.0), cmul(pm, e0.s0)), a1 = cscale(kh * (-r + 1.0), cmul(pm, e0.s1));
  const double2 b0 = cscale(kh * (-r + 1.0), cmul(pp, e1.s0)), b1 = cscale(kh * (-r - 1.0), cmul(pp, e1.s1));
  auto re_ci = [](double2 a, double2 b) { return a.y * b.x - a.x * b.y; };  // Re[conj(a) (i b)]
  // (D eta)_{s+1}^dag (-i a) = -Re[conj(d1) (i a)];  (D eta)_s^dag (i b)
  const double inner = -(re_ci(d1.s0, a0) + re_ci(d1.s1, a1)) + re_ci(d0.s0, b0) + re_ci(d0.s1, b1);
  double& o = F[size_t(Nt) * Nl + size_t(s) * Ns + x];
  o = acc ? o + c * (-2.0 * inner) : c * (-2.0 * inner);
}

int ext_init(qed3_dirac_ext_s* e) {
  qed3_dirac_s* d = e->d2;
  const HostLattice& L = d->lat->host;
  const int Ns = d->Ns, Nt = e->Nt;
  // per-site tables in reference order (the apply's thread order)
  std::vector<double> kt(Ns), diag2(Ns), diag3(Ns);
  std::vector<int32_t> nbr(size_t(3) * Ns), nbrR(size_t(3) * Ns);
  QED3_CUDA_TRY(cudaMemcpy(diag2.data(), d->diag, Ns * sizeof(double), cudaMemcpyDeviceToHost));
  QED3_CUDA_TRY(cudaMemcpy(nbr.data(), d->lat->dev.nbr_ref, nbr.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
  for (int i = 0; i < Ns; i++) {
    const int x = L.perm[i];
    kt[x] = Nt != 1 ? L.tri_area[x] / L.mean_ell / e->at : 0.0;
    diag3[x] = diag2[i] + e->r * kt[x];
    for (int k = 0; k < 3; k++) nbrR[size_t(k) * Ns + x] = nbr[size_t(k) * Ns + i];
  }
  const size_t nh = size_t(3) * Ns * Nt;
  QED3_CUDA_TRY(cudaMalloc(&e->H3, nh * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&e->Hd3, nh * sizeof(M64)));
  QED3_CUDA_TRY(cudaMalloc(&e->kt, Ns * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&e->diag3, Ns * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&e->Pt, size_t(Ns) * Nt * sizeof(double2)));
  QED3_CUDA_TRY(cudaMalloc(&e->nbrR, nbrR.size() * sizeof(int32_t)));
  QED3_CUDA_TRY(cudaMemcpy(e->nbrR, nbrR.data(), nbrR.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMalloc(&e->tmp, size_t(Ns) * Nt * sizeof(S64)));
  // CG vectors, then 2048 doubles of reduction partials (vec_zdot fills all of
  // them on large fields), then the device-resident CG state
  QED3_CUDA_TRY(cudaMalloc(&e->work, size_t(Ns) * Nt * 3 * sizeof(S64) + (2048 + 64) * sizeof(double)));
  QED3_CUDA_TRY(cudaMemcpy(e->kt, kt.data(), Ns * sizeof(double), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(e->diag3, diag3.data(), Ns * sizeof(double), cudaMemcpyHostToDevice));
  return QED3_OK;
}

void ext_free(qed3_dirac_ext_s* e) {
  void* p[] = {e->H3, e->Hd3, e->kt, e->diag3, e->Pt, e->nbrR, e->tmp, e->work, e->H3f, e->Hd3f, e->Ptf, e->diag3f,
               e->ktf, e->fwork};
  for (void* q : p)
    if (q) cudaFree(q);
}

int ext_set_links(qed3_dirac_ext_s* e, const double* A, cudaStream_t st) {
  qed3_dirac_s* d = e->d2;
  const DeviceLattice& D = d->lat->dev;
  const int Ns = d->Ns, Nl = D.Nl, Nt = e->Nt;
  k_ext_set_links<<<nblk(4LL * Ns * Nt), 256, 0, st>>>(Ns, Nl, Nt, D.iperm, D.hop_link, D.hop_sign, A, d->G, d->Gd,
                                                      e->H3, e->Hd3, e->Pt);
  QED3_CUDA_TRY(cudaGetLastError());
  e->links_set = true;
  e->f32_current = false;
  return QED3_OK;
}

int ext_apply(qed3_dirac_ext_s* e, int op, double* out, const double* in, cudaStream_t st) {
  if (!e->links_set) return fail(QED3_ERR_STATE, "call qed3_dirac_ext_set_links first");
  qed3_dirac_s* d = e->d2;
  const DeviceLattice& D = d->lat->dev;
  const int Ns = d->Ns, Nt = e->Nt;
  const long long n = (long long)Ns * Nt;
  auto run = [&](int adj, S64* o, const S64* v) {
    k_ext_apply<<<nblk(n), 256, 0, st>>>(Ns, Nt, adj, e->nbrR, adj ? e->Hd3 : e->H3, e->diag3, e->kt, e->Pt, d->r,
                                        v, o);
  };
  const S64* v = reinterpret_cast<const S64*>(in);
  S64* o = reinterpret_cast<S64*>(out);
  if (op == QED3_OP_D || op == QED3_OP_DDAG) {
    if (in == out) {
      QED3_CUDA_TRY(cudaMemcpyAsync(e->tmp, in, n * sizeof(S64), cudaMemcpyDeviceToDevice, st));
      v = e->tmp;
    }
    run(op == QED3_OP_DDAG, o, v);
  } else if (op == QED3_OP_DDAGD) {
    run(0, e->tmp, v);
    run(1, o, e->tmp);
  } else if (op == QED3_OP_DDDAG) {
    run(1, e->tmp, v);
    run(0, o, e->tmp);
  } else {
    return fail(QED3_ERR_ARG, "unknown operator");
  }
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// F (+)= c (-2 Re <chi, dD/dA eta>) for every spatial and temporal link
int ext_force_bilinear(qed3_dirac_ext_s* e, const double* chi, const double* eta, double c, int acc, double* F,
                       cudaStream_t st) {
  qed3_dirac_s* d = e->d2;
  const DeviceLattice& D = d->lat->dev;
  const int Ns = d->Ns, Nl = D.Nl, Nt = e->Nt;
  const S64* et = reinterpret_cast<const S64*>(eta);
  const S64* ch = reinterpret_cast<const S64*>(chi);
  k_ext_force_sp<<<nblk((long long)Nl * Nt), 256, 0, st>>>(Ns, Nl, Nt, D.link_x, D.link_y, D.link_kx, D.link_ky, D.perm,
                                                          e->H3, et, ch, c, acc, F);
  if (Nt > 1)
    k_ext_force_tp<<<nblk((long long)Ns * Nt), 256, 0, st>>>(Ns, Nl, Nt, e->kt, e->Pt, d->r, et, ch, c, acc, F);
  else if (!acc)
    QED3_CUDA_TRY(cudaMemsetAsync(F + size_t(Nt) * Nl, 0, size_t(Ns) * sizeof(double), st));
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int ext_fermion_force(qed3_dirac_ext_s* e, const double* eta, double* F, cudaStream_t st) {
  if (!e->links_set) return fail(QED3_ERR_STATE, "call qed3_dirac_ext_set_links first");
  double* deta = reinterpret_cast<double*>(e->work);  // D eta (the CG vectors are not in use here)
  int rc = ext_apply(e, QED3_OP_D, deta, eta, st);
  if (rc) return rc;
  return ext_force_bilinear(e, deta, eta, 1.0, 0, F, st);
}

// ---- CG with device-resident scalars ------------------------------------------
// alpha, beta and the residual norm stay on the device: one iteration is the
// operator and five small kernels, with no host round trip.  Once the
// recursive residual meets the tolerance (or turns non-finite) the state's
// `done` flag makes the remaining kernels of the launched chunk return at
// once, so the iterate and the iteration count are those of the host-driven
// recurrence; the host reads the state once per chunk.
struct ExtCgState {
  double mu, thr, alpha, beta, done, iters;  // done: 0 running, 1 converged, 2 non-finite
};
constexpr int kCgParts = 304;  // partial sums: two blocks per SM


__global__ void k_cg_pq(long long nc, const double2* __restrict__ p, const double2* __restrict__ q,
                        double* __restrict__ part, const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    const double2 a = p[i], b = q[i];
    v[0] += a.x * b.x + a.y * b.y;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// alpha = mu / Re<p, A p> (one block; fixed summation order)
__global__ void k_cg_alpha(const double* __restrict__ part, int np, ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < np; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) stt->alpha = stt->mu / v[0];
}

// x += alpha p, r -= alpha q, partial sums of |r|^2
__global__ void k_cg_xr(long long nc, const double2* __restrict__ p, const double2* __restrict__ q,
                        double2* __restrict__ x, double2* __restrict__ r, double* __restrict__ part,
                        const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  const double al = stt->alpha;
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    const double2 pp = p[i], qq = q[i];
    double2 xx = x[i], rr = r[i];
    xx.x += al * pp.x;
    xx.y += al * pp.y;
    rr.x -= al * qq.x;
    rr.y -= al * qq.y;
    x[i] = xx;
    r[i] = rr;
    v[0] += rr.x * rr.x + rr.y * rr.y;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// |r|^2, the stopping test, beta = |r|^2 / mu
__global__ void k_cg_beta(const double* __restrict__ part, int np, ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < np; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) {
    const double mn = v[0];
    stt->iters += 1.0;
    if (!isfinite(mn)) {
      stt->done = 2.0;
    } else if (mn < stt->thr) {
      stt->done = 1.0;
    } else {
      stt->beta = mn / stt->mu;
      stt->mu = mn;
    }
  }
}

__global__ void k_cg_p(long long nc, const double2* __restrict__ r, double2* __restrict__ p,
                       const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  const double bt = stt->beta;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
    const double2 rr = r[i], pp = p[i];
    p[i] = make_double2(rr.x + bt * pp.x, rr.y + bt * pp.y);
  }
}

// ---- FP32 operator and the mixed-precision CG ------------------------------
// GB300's FP64 pipe bounds the FP64 apply (it runs at ~92 % of that pipe);
// the FP32 copy of the operator moves half the bytes through the wide FP32
// pipe.  The CG iterates in FP32 on the residual scaled to unit norm, and
// every time that residual has dropped by delta (or meets the tolerance) the
// FP64 solution and the FP64 true residual b - A x are refreshed (reliable
// update); the search direction is kept, rescaled to the new residual norm.
__global__ void k_ext_to32(long long nh, long long np, const M64* __restrict__ H3, const M64* __restrict__ Hd3,
                           const double2* __restrict__ Pt, M32* __restrict__ H3f, M32* __restrict__ Hd3f,
                           float2* __restrict__ Ptf) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  auto cv = [](const M64& h) {
    return M32{make_float4(float(h.h00.x), float(h.h00.y), float(h.h01.x), float(h.h01.y)),
               make_float4(float(h.h10.x), float(h.h10.y), float(h.h11.x), float(h.h11.y))};
  };
  if (idx < nh) {
    H3f[idx] = cv(H3[idx]);
    Hd3f[idx] = cv(Hd3[idx]);
  } else if (idx - nh < np) {
    const double2 p = Pt[idx - nh];
    Ptf[idx - nh] = make_float2(float(p.x), float(p.y));
  }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// k_ext_apply in FP32 (same entries, same thread order)
__global__ void k_ext_apply32(int Ns, int Nt, int adj, const int32_t* __restrict__ nbrR, const M32* __restrict__ H3,
                              const float* __restrict__ diag3, const float* __restrict__ kt,
                              const float2* __restrict__ Pt, float r, const float4* __restrict__ in,
                              float4* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Ns * Nt) return;
  const int s = int(idx / Ns), x = int(idx % Ns);
  const float4* vs = in + size_t(s) * Ns;
  const Sp32 self = ld32(vs, x);
  const float dg = diag3[x];
  Sp32 o{make_float2(dg * self.s0.x, dg * self.s0.y), make_float2(dg * self.s1.x, dg * self.s1.y)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const M32 m = H3[(size_t(s) * 3 + k) * Ns + x];
    const Sp32 b = ld32(vs, nbrR[size_t(k) * Ns + x]);
    o.s0 = cfmaf(make_float2(m.r0.x, m.r0.y), b.s0, o.s0);
    o.s0 = cfmaf(make_float2(m.r0.z, m.r0.w), b.s1, o.s0);
    o.s1 = cfmaf(make_float2(m.r1.x, m.r1.y), b.s0, o.s1);
    o.s1 = cfmaf(make_float2(m.r1.z, m.r1.w), b.s1, o.s1);
  }
  if (Nt > 1) {
    const float kh = 0.5f * kt[x];
    const int sp = (s + 1) % Nt, sm = (s + Nt - 1) % Nt;
    const Sp32 up = ld32(in + size_t(sp) * Ns, x), dn = ld32(in + size_t(sm) * Ns, x);
    float cu0, cu1, cd0, cd1;
    if (!adj) {
      const float sgn_u = (sp == 0) ? -1.f : 1.f, sgn_d = (sm == Nt - 1) ? -1.f : 1.f;
      cu0 = sgn_u * kh * (-r + 1.f);
      cu1 = sgn_u * kh * (-r - 1.f);
      cd0 = sgn_d * kh * (-r - 1.f);
      cd1 = sgn_d * kh * (-r + 1.f);
    } else {
      const float sgn_u = (s == Nt - 1) ? -1.f : 1.f, sgn_d = (s == 0) ? -1.f : 1.f;
      cu0 = sgn_u * kh * (-r - 1.f);
      cu1 = sgn_u * kh * (-r + 1.f);
      cd0 = sgn_d * kh * (-r + 1.f);
      cd1 = sgn_d * kh * (-r - 1.f);
    }
    const float2 pu = Pt[size_t(s) * Ns + x], pdc = Pt[size_t(sm) * Ns + x];
    const float2 pd = make_float2(pdc.x, -pdc.y);
    const float2 u0 = cmulf(pu, up.s0), u1 = cmulf(pu, up.s1), d0 = cmulf(pd, dn.s0), d1 = cmulf(pd, dn.s1);
    o.s0.x += cu0 * u0.x + cd0 * d0.x;
    o.s0.y += cu0 * u0.y + cd0 * d0.y;
    o.s1.x += cu1 * u1.x + cd1 * d1.x;
    o.s1.y += cu1 * u1.y + cd1 * d1.y;
  }
  st32(out + size_t(s) * Ns, x, o);
}

// Re<p, q> partial sums (FP32 vectors, FP64 accumulation)
__global__ void k_mcg_pq(long long n, const float4* __restrict__ p, const float4* __restrict__ q,
                         double* __restrict__ part, const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 a = p[i], b = q[i];
    v[0] += double(a.x) * b.x + double(a.y) * b.y + double(a.z) * b.z + double(a.w) * b.w;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_mcg_xr(long long n, const float4* __restrict__ p, const float4* __restrict__ q,
                         float4* __restrict__ x, float4* __restrict__ r, double* __restrict__ part,
                         const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  __shared__ double sh[32];
  const float al = float(stt->alpha);
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 pp = p[i], qq = q[i];
    float4 xx = x[i], rr = r[i];
    xx.x += al * pp.x; xx.y += al * pp.y; xx.z += al * pp.z; xx.w += al * pp.w;
    rr.x -= al * qq.x; rr.y -= al * qq.y; rr.z -= al * qq.z; rr.w -= al * qq.w;
    x[i] = xx;
    r[i] = rr;
    v[0] += double(rr.x) * rr.x + double(rr.y) * rr.y + double(rr.z) * rr.z + double(rr.w) * rr.w;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_mcg_p(long long n, const float4* __restrict__ r, float4* __restrict__ p,
                        const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  const float bt = float(stt->beta);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 rr = r[i], pp = p[i];
    p[i] = make_float4(rr.x + bt * pp.x, rr.y + bt * pp.y, rr.z + bt * pp.z, rr.w + bt * pp.w);
  }
}

__global__ void k_mcg_shift(long long n, float sh, const float4* __restrict__ p, float4* __restrict__ q,
                            const ExtCgState* __restrict__ stt) {
  if (stt->done != 0.0) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 pp = p[i];
    float4 qq = q[i];
    qq.x += sh * pp.x; qq.y += sh * pp.y; qq.z += sh * pp.z; qq.w += sh * pp.w;
    q[i] = qq;
  }
}

// reliable update, part 1: x += sigma xf (FP64), xf = 0
__global__ void k_mcg_accum(long long n, double sigma, float4* __restrict__ xf, S64* __restrict__ x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 a = xf[i];
    S64 v = x[i];
    v.s0.x += sigma * double(a.x);
    v.s0.y += sigma * double(a.y);
    v.s1.x += sigma * double(a.z);
    v.s1.y += sigma * double(a.w);
    x[i] = v;
    xf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// reliable update, part 2: rf = r / sigma, p *= pscale, partial |rf|^2
__global__ void k_mcg_restart(long long n, double sinv, float pscale, const S64* __restrict__ r,
                              float4* __restrict__ rf, float4* __restrict__ pf, double* __restrict__ part) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const S64 a = r[i];
    const float4 f = make_float4(float(a.s0.x * sinv), float(a.s0.y * sinv), float(a.s1.x * sinv), float(a.s1.y * sinv));
    rf[i] = f;
    float4 pp = pf[i];
    pp.x *= pscale; pp.y *= pscale; pp.z *= pscale; pp.w *= pscale;
    pf[i] = pp;
    v[0] += double(f.x) * f.x + double(f.y) * f.y + double(f.z) * f.z + double(f.w) * f.w;
  }
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// reliable update, part 3: mu = |rf|^2, new threshold, running again
__global__ void k_mcg_setmu(const double* __restrict__ part, int np, double thr, ExtCgState* __restrict__ stt) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < np; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) {
    stt->mu = v[0];
    stt->thr = thr;
    stt->done = 0.0;
  }
}

static int ext_ensure_f32(qed3_dirac_ext_s* e, cudaStream_t st) {
  const int Ns = e->d2->Ns, Nt = e->Nt;
  const size_t nh = size_t(3) * Ns * Nt, np = size_t(Ns) * Nt;
  if (!e->H3f) {
    std::vector<double> kt(Ns), dg(Ns);
    QED3_CUDA_TRY(cudaMemcpy(kt.data(), e->kt, Ns * sizeof(double), cudaMemcpyDeviceToHost));
    QED3_CUDA_TRY(cudaMemcpy(dg.data(), e->diag3, Ns * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<float> ktf(kt.begin(), kt.end()), dgf(dg.begin(), dg.end());
    QED3_CUDA_TRY(cudaMalloc(&e->H3f, nh * sizeof(M32)));
    QED3_CUDA_TRY(cudaMalloc(&e->Hd3f, nh * sizeof(M32)));
    QED3_CUDA_TRY(cudaMalloc(&e->Ptf, np * sizeof(float2)));
    QED3_CUDA_TRY(cudaMalloc(&e->diag3f, Ns * sizeof(float)));
    QED3_CUDA_TRY(cudaMalloc(&e->ktf, Ns * sizeof(float)));
    QED3_CUDA_TRY(cudaMalloc(&e->fwork, 5 * np * sizeof(float4)));
    QED3_CUDA_TRY(cudaMemcpy(e->ktf, ktf.data(), Ns * sizeof(float), cudaMemcpyHostToDevice));
    QED3_CUDA_TRY(cudaMemcpy(e->diag3f, dgf.data(), Ns * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (!e->f32_current) {
    k_ext_to32<<<nblk((long long)(nh + np)), 256, 0, st>>>((long long)nh, (long long)np, e->H3, e->Hd3, e->Pt, e->H3f,
                                                          e->Hd3f, e->Ptf);
    QED3_CUDA_TRY(cudaGetLastError());
    e->f32_current = true;
  }
  return QED3_OK;
}

static int ext_cg_mixed(qed3_dirac_ext_s* e, double* x, const double* b, double tol, int maxiter, double shift,
                        double delta, qed3_solve_report* rep, cudaStream_t st, int op) {
  int rc = ext_ensure_f32(e, st);
  if (rc) return rc;
  const int Ns = e->d2->Ns, Nt = e->Nt;
  const long long n = (long long)Ns * Nt, nd = 4 * n, nc = 2 * n;
  double* r = reinterpret_cast<double*>(e->work);
  double* q = r + 2 * nd;
  double* part = q + nd;
  float4 *rf = e->fwork, *pf = rf + n, *qf = pf + n, *tf = qf + n, *xf = tf + n;
  EventPair ev;
  QED3_CUDA_TRY(ev.create());
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  QED3_CUDA_TRY(cudaEventRecord(e0, st));
  auto A64 = [&](double* o, const double* v) -> int {
    int c = ext_apply(e, op, o, v, st);
    if (!c && shift != 0.0) c = vec_axpby(nd, shift, v, 1.0, o, o, st);
    return c;
  };
  const int gs = nblk(n);
  const int first = op == QED3_OP_DDAGD ? 0 : 1;  // D^dag D: D then D^dag; D D^dag: the reverse
  auto A32 = [&](float4* o, const float4* v, cudaStream_t s) {
    k_ext_apply32<<<gs, 256, 0, s>>>(Ns, Nt, first, e->nbrR, first ? e->Hd3f : e->H3f, e->diag3f, e->ktf, e->Ptf,
                                     float(e->r), v, tf);
    k_ext_apply32<<<gs, 256, 0, s>>>(Ns, Nt, 1 - first, e->nbrR, first ? e->H3f : e->Hd3f, e->diag3f, e->ktf,
                                     e->Ptf, float(e->r), tf, o);
  };
  double bb = 0, im = 0;
  if ((rc = vec_zdot(nc, b, b, part, &bb, &im, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(x, 0, nd * sizeof(double), st));
  QED3_CUDA_TRY(cudaMemsetAsync(xf, 0, n * sizeof(float4), st));
  QED3_CUDA_TRY(cudaMemsetAsync(pf, 0, n * sizeof(float4), st));
  ExtCgState* dst = reinterpret_cast<ExtCgState*>(part + 2048);
  ExtCgState hst{0.0, 0.0, 0.0, 0.0, bb == 0.0 ? 1.0 : 0.0, 0.0};
  QED3_CUDA_TRY(cudaMemcpyAsync(dst, &hst, sizeof(hst), cudaMemcpyHostToDevice, st));
  const int gblk = int(std::min<long long>(kCgParts, (n + 255) / 256));
  int status = bb == 0.0 ? QED3_OK : QED3_ERR_NOCONV, updates = 0, its = 0;
  double rr = bb, sigma = 0.0;
  // (re)start the FP32 iteration on r / |r|: p = r / |r| at the start, p rescaled later
  auto restart = [&](double rr_now, bool first_time) -> int {
    const double snew = std::sqrt(rr_now);
    const float pscale = first_time ? 0.f : float(sigma / snew);
    k_mcg_restart<<<gblk, 256, 0, st>>>(n, 1.0 / snew, pscale, reinterpret_cast<const S64*>(r), rf, pf, part);
    if (first_time) QED3_CUDA_TRY(cudaMemcpyAsync(pf, rf, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    k_mcg_setmu<<<1, 256, 0, st>>>(part, gblk, tol * tol * bb / rr_now, dst);
    QED3_CUDA_TRY(cudaGetLastError());
    sigma = snew;
    return QED3_OK;
  };
  if (bb > 0) {
    QED3_CUDA_TRY(cudaMemcpyAsync(r, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if ((rc = restart(bb, true))) return rc;
  }
  const double d2 = delta * delta;
  auto iter = [&](cudaStream_t s) -> int {
    A32(qf, pf, s);
    if (shift != 0.0) k_mcg_shift<<<gblk, 256, 0, s>>>(n, float(shift), pf, qf, dst);
    k_mcg_pq<<<gblk, 256, 0, s>>>(n, pf, qf, part, dst);
    k_cg_alpha<<<1, 256, 0, s>>>(part, gblk, dst);
    k_mcg_xr<<<gblk, 256, 0, s>>>(n, pf, qf, xf, rf, part, dst);
    k_cg_beta<<<1, 256, 0, s>>>(part, gblk, dst);
    k_mcg_p<<<gblk, 256, 0, s>>>(n, rf, pf, dst);
    return QED3_OK;
  };
  const int chunk = 8;
  IterGraph graph;
  const bool use_graph = status != QED3_OK && maxiter >= chunk && graph.build(chunk, iter);
  while (status != QED3_OK && its < maxiter) {
    const int m = std::min(chunk, maxiter - its);
    if (use_graph && m == chunk) {
      QED3_CUDA_TRY(cudaGraphLaunch(graph.exec, st));
    } else {
      for (int k = 0; k < m; k++) iter(st);
    }
    QED3_CUDA_TRY(cudaGetLastError());
    QED3_CUDA_TRY(cudaMemcpyAsync(&hst, dst, sizeof(hst), cudaMemcpyDeviceToHost, st));
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
    its = int(hst.iters);
    if (hst.done == 2.0) break;  // non-finite
    // the scaled residual norm: |r|^2 / sigma^2 after the last completed step
    if (hst.done == 1.0 || hst.mu < d2 || its >= maxiter) {
      k_mcg_accum<<<gblk, 256, 0, st>>>(n, sigma, xf, reinterpret_cast<S64*>(x));
      QED3_CUDA_TRY(cudaGetLastError());
      if ((rc = A64(q, x)) || (rc = vec_axpby(nd, 1.0, b, -1.0, q, r, st)) ||
          (rc = vec_zdot(nc, r, r, part, &rr, &im, st)))
        return rc;
      updates++;
      if (!std::isfinite(rr)) break;
      if (rr < tol * tol * bb) {
        status = QED3_OK;
        break;
      }
      if (its >= maxiter) break;
      if ((rc = restart(rr, false))) return rc;
    }
  }
  QED3_CUDA_TRY(cudaEventRecord(e1, st));
  QED3_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (rep) {
    rep->status = status;
    rep->iters = its;
    rep->reliable_updates = updates;
    rep->true_rel_res = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    rep->ms = ms;
  }
  return QED3_OK;
}

// MatPoly::solve (src/dual/matpoly.h:204-267) on D^dag D + shift in FP64:
// x0 = 0, stop on the recursive residual, certified by the true residual.
// precision QED3_PREC_F32: the mixed-precision CG above (same certificate).
int ext_cg(qed3_dirac_ext_s* e, double* x, const double* b, const qed3_solve_params* prm, qed3_solve_report* rep,
           cudaStream_t st, int op) {
  if (op != QED3_OP_DDAGD && op != QED3_OP_DDDAG) return fail(QED3_ERR_ARG, "CG runs on D^dag D or D D^dag");
  if (!e->links_set) return fail(QED3_ERR_STATE, "call qed3_dirac_ext_set_links first");
  if (prm && prm->precision == QED3_PREC_F32)
    return ext_cg_mixed(e, x, b, prm->tol > 0 ? prm->tol : 1e-10, prm->maxiter > 0 ? prm->maxiter : 100000,
                        prm->shift, prm->delta > 0 && prm->delta < 1 ? prm->delta : 0.1, rep, st, op);
  if (prm && prm->precision != QED3_PREC_F64) return fail(QED3_ERR_ARG, "the S2 x S1 solve runs in FP64 or FP32");
  const double tol = prm && prm->tol > 0 ? prm->tol : 1e-10;
  const int maxiter = prm && prm->maxiter > 0 ? prm->maxiter : 100000;
  const double shift = prm ? prm->shift : 0.0;
  const long long nd = 4LL * e->d2->Ns * e->Nt, nc = nd / 2;
  double* r = reinterpret_cast<double*>(e->work);
  double* p = r + nd;
  double* q = p + nd;
  double* part = q + nd;
  EventPair ev;
  QED3_CUDA_TRY(ev.create());
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  QED3_CUDA_TRY(cudaEventRecord(e0, st));
  auto As = [&](double* o, const double* v, cudaStream_t s) -> int {
    int c = ext_apply(e, op, o, v, s);
    if (!c && shift != 0.0) c = vec_axpby(nd, shift, v, 1.0, o, o, s);
    return c;
  };
  auto A = [&](double* o, const double* v) -> int { return As(o, v, st); };
  int rc;
  double bb = 0, im = 0;
  if ((rc = vec_zdot(nc, b, b, part, &bb, &im, st))) return rc;
  QED3_CUDA_TRY(cudaMemsetAsync(x, 0, nd * sizeof(double), st));
  QED3_CUDA_TRY(cudaMemcpyAsync(r, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(p, b, nd * sizeof(double), cudaMemcpyDeviceToDevice, st));
  ExtCgState* dst = reinterpret_cast<ExtCgState*>(part + 2048);
  ExtCgState hst{bb, tol * tol * bb, 0.0, 0.0, bb == 0.0 ? 1.0 : 0.0, 0.0};
  QED3_CUDA_TRY(cudaMemcpyAsync(dst, &hst, sizeof(hst), cudaMemcpyHostToDevice, st));
  const double2* p2 = reinterpret_cast<const double2*>(p);
  const double2* q2 = reinterpret_cast<const double2*>(q);
  const int gblk = int(std::min<long long>(kCgParts, (nc + 255) / 256));
  int launched = 0;
  const int chunk = 16;
  auto iter = [&](cudaStream_t s) -> int {
    const int c = As(q, p, s);
    if (c) return c;
    k_cg_pq<<<gblk, 256, 0, s>>>(nc, p2, q2, part, dst);
    k_cg_alpha<<<1, 256, 0, s>>>(part, gblk, dst);
    k_cg_xr<<<gblk, 256, 0, s>>>(nc, p2, q2, reinterpret_cast<double2*>(x), reinterpret_cast<double2*>(r), part, dst);
    k_cg_beta<<<1, 256, 0, s>>>(part, gblk, dst);
    k_cg_p<<<gblk, 256, 0, s>>>(nc, reinterpret_cast<const double2*>(r), reinterpret_cast<double2*>(p), dst);
    return QED3_OK;
  };
  IterGraph graph;
  const bool use_graph = hst.done == 0.0 && maxiter >= chunk && graph.build(chunk, iter);
  while (hst.done == 0.0 && launched < maxiter) {
    const int m = std::min(chunk, maxiter - launched);
    if (use_graph && m == chunk) {
      QED3_CUDA_TRY(cudaGraphLaunch(graph.exec, st));
    } else {
      for (int k = 0; k < m; k++)
        if ((rc = iter(st))) return rc;
    }
    QED3_CUDA_TRY(cudaGetLastError());
    launched += m;
    QED3_CUDA_TRY(cudaMemcpyAsync(&hst, dst, sizeof(hst), cudaMemcpyDeviceToHost, st));
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
  }
  const int it = int(hst.iters);
  const int status = hst.done == 1.0 ? QED3_OK : QED3_ERR_NOCONV;
  double tr = 0;
  if (bb > 0) {
    if ((rc = A(q, x)) || (rc = vec_axpby(nd, 1.0, b, -1.0, q, q, st)) || (rc = vec_zdot(nc, q, q, part, &tr, &im, st)))
      return rc;
  }
  QED3_CUDA_TRY(cudaEventRecord(e1, st));
  QED3_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (rep) {
    rep->status = status;
    rep->iters = it;
    rep->reliable_updates = 0;
    rep->true_rel_res = bb > 0 ? std::sqrt(tr / bb) : 0.0;
    rep->ms = ms;
  }
  return QED3_OK;
}

}  // namespace qed3

// ===========================================================================
// S^2 x S^1 HMC trajectory: HMC2::run (src/both_3d/hmc.h:172-200) with the
// anisotropic gauge action U1WilsonExt and npf Wilson pseudofermions of the
// DiracExt operator, ExplicitLeapfrogML (src/both_3d/integrator.h:117-168) or
// ExplicitLeapfrog.  The random streams are ParallelRngExt's: link engines
// [Nt][Nl], site engines [Nt][Ns] (qed3_rng_create(Nt Nl, Nt Ns, seed));
// momenta: spatial from the link engines, temporal one per site engine
// (GaugeExt::gaussian); xi = fill_gaussian from the site engines.
// H = |pi|^2 / 2 + S_g + sum Re <phi, eta>, dH = H1 - H0 as the reference.
// ===========================================================================
#include "gauge_impl.h"

namespace qed3 {

int hmc_ext(qed3_dirac_ext_s* e, qed3_rng_s* rng, double* A, double at, double gsq, double tmax, int nsteps,
            int nsteps_inner, int npf, int integrator, double tol, int prec, int no_reject, int* accepted,
            double* dH_out, int* cg_iters, cudaStream_t st, qed3_overlap_ext_s* ov, double tol_inner, double lmin_fix,
            double lmax_fix) {
  qed3_dirac_s* d = e->d2;
  qed3_lattice_s* lat = d->lat;
  const int Ns = d->Ns, Nl = lat->dev.Nl, Nt = e->Nt;
  const long long nA = (long long)Nt * (Nl + Ns), nd = 4LL * Ns * Nt;
  std::vector<double> pi(static_cast<size_t>(nA)), xi(static_cast<size_t>(nd * npf));
  rng_gaussian_links(rng, 1.0, pi.data());
  rng_gaussian_sites(rng, 1.0, pi.data() + size_t(Nt) * Nl);
  for (int k = 0; k < npf; k++) rng_gaussian_spinor(rng, xi.data() + nd * k);
  double* buf = nullptr;
  const size_t bytes = (size_t(nA) * 4 + size_t(nd) * npf * 3 + 2048) * sizeof(double);
  if (cudaMalloc(&buf, bytes) != cudaSuccess) return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  double *P = buf, *A0 = P + nA, *F = A0 + nA, *Ff = F + nA, *xid = Ff + nA, *phi = xid + nd * npf,
         *eta = phi + nd * npf, *part = eta + nd * npf;
  int its = 0;
  const qed3_solve_params sp{tol, 0, prec, 0.1, 0.0, 0};
  auto body = [&]() -> int {
    int rc;
    QED3_CUDA_TRY(cudaMemcpyAsync(P, pi.data(), nA * sizeof(double), cudaMemcpyHostToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(A0, A, nA * sizeof(double), cudaMemcpyDeviceToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(xid, xi.data(), nd * npf * sizeof(double), cudaMemcpyHostToDevice, st));
    // the fermion operator: the Wilson DiracExt, or its overlap (Overlap::update
    // recomputes the bounds at every link update unless they are fixed)
    auto update_op = [&]() -> int {
      int c = ext_set_links(e, A, st);
      if (!c && ov) c = ext_overlap_update(ov, lmin_fix, lmax_fix, 1e-10, 1e-6, st);
      return c;
    };
    if ((rc = update_op())) return rc;
    for (int k = 0; k < npf; k++)
      if ((rc = ov ? ext_overlap_apply(ov, QED3_OP_DDAG, phi + nd * k, xid + nd * k, tol_inner, nullptr, st)
                   : ext_apply(e, QED3_OP_DDAG, phi + nd * k, xid + nd * k, st)))
        return rc;
    auto solve_all = [&]() -> int {
      for (int k = 0; k < npf; k++) {
        qed3_solve_report r{};
        int c = ov ? ext_overlap_solve(ov, eta + nd * k, phi + nd * k, tol, tol_inner, 100000, 0, &r, st)
                   : ext_cg(e, eta + nd * k, phi + nd * k, &sp, &r, st);
        its += r.iters;
        if (!c && r.status != QED3_OK) c = fail(QED3_ERR_NOCONV, "pseudofermion solve did not converge");
        if (c) return c;
      }
      return QED3_OK;
    };
    auto H = [&](double* h) -> int {
      double kin = 0, im = 0, sg = 0, sf = 0;
      int c = vec_zdot(nA / 2, P, P, part, &kin, &im, st);  // nA is even: Nt (Nl + Ns) with Nl, Ns even
      if (c) return c;
      if ((c = ext_gauge_action(lat, Nt, at, gsq, A, &sg, st))) return c;
      for (int k = 0; k < npf; k++) {
        double re = 0;
        if ((c = vec_zdot(nd / 2, phi + nd * k, eta + nd * k, part, &re, &im, st))) return c;
        sf += re;
      }
      *h = 0.5 * kin + sg + sf;
      return QED3_OK;
    };
    if ((rc = solve_all())) return rc;
    double h0 = 0, h1 = 0;
    if ((rc = H(&h0))) return rc;
    const double tau = tmax / nsteps, tau_in = tau / nsteps_inner;
    auto gauge_kick = [&](double c) -> int {
      int q = ext_gauge_force(lat, Nt, at, gsq, A, F, st);
      return q ? q : vec_axpby(nA, -c, F, 1.0, P, P, st);
    };
    auto ferm_force = [&](int k) -> int {
      return ov ? ext_overlap_force(ov, eta + nd * k, Ff, tol_inner, nullptr, st)
                : ext_fermion_force(e, eta + nd * k, Ff, st);
    };
    auto fermion_kick = [&](int k, double c) -> int {
      int q = ferm_force(k);
      return q ? q : vec_axpby(nA, -c, Ff, 1.0, P, P, st);
    };
    auto full_kick = [&](double c) -> int {  // pi += -c (dSg + dSf)
      int q = ext_gauge_force(lat, Nt, at, gsq, A, F, st);
      for (int k = 0; k < npf && !q; k++) {
        q = ferm_force(k);
        if (!q) q = vec_axpby(nA, 1.0, Ff, 1.0, F, F, st);
      }
      return q ? q : vec_axpby(nA, -c, F, 1.0, P, P, st);
    };
    auto drift = [&](double c) -> int { return vec_axpby(nA, c, P, 1.0, A, A, st); };
    if (integrator == QED3_INTEGRATOR_LEAPFROG) {
      for (int n = 0; n < nsteps; n++) {
        if ((rc = full_kick(0.5 * tau)) || (rc = drift(tau)) || (rc = update_op()) ||
            (rc = solve_all()) || (rc = full_kick(0.5 * tau)))
          return rc;
      }
    } else {
      for (int k = 0; k < npf; k++)
        if ((rc = fermion_kick(k, 0.5 * tau))) return rc;
      for (int n = 0; n < nsteps; n++) {
        if ((rc = gauge_kick(0.5 * tau_in))) return rc;
        for (int m = 0; m < nsteps_inner; m++)
          if ((rc = drift(tau_in)) || (rc = gauge_kick((m != nsteps_inner - 1 ? 1.0 : 0.5) * tau_in))) return rc;
        if ((rc = update_op()) || (rc = solve_all())) return rc;
        for (int k = 0; k < npf; k++)
          if ((rc = fermion_kick(k, (n != nsteps - 1 ? 1.0 : 0.5) * tau))) return rc;
      }
    }
    if ((rc = H(&h1))) return rc;
    const double dH = h1 - h0;
    *dH_out = dH;
    if (cg_iters) *cg_iters = its;
    const double r = std::min(1.0, std::exp(-dH));
    const double a = rng_uniform(rng);
    if (a < r || no_reject) {
      *accepted = 1;
    } else {
      *accepted = 0;
      QED3_CUDA_TRY(cudaMemcpyAsync(A, A0, nA * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if ((rc = update_op())) return rc;
    }
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
    return QED3_OK;
  };
  const int rc = body();
  cudaFree(buf);
  return rc;
}

}  // namespace qed3

namespace qed3 {

// Point-source propagator of prop.cu (src/both_3d/prop.cu:243-268):
// src1 = delta at (slice s, site ix, spin a) (FermionVector::set_pt_source,
// src/both_3d/valence.h:67-72), src = D^dag src1, sink = (D^dag D)^{-1} src
// = D^{-1} src1 by the FP64 CG; dagger (IS_DAGGER): src = D src1, sink =
// (D D^dag)^{-1} src = D^{-dag} src1.  Site ix in the reference's numbering.
int ext_propagator(qed3_dirac_ext_s* e, int s, int ix, int a, int dagger, double* sink, const qed3_solve_params* prm,
                   qed3_solve_report* rep, cudaStream_t st) {
  if (!e->links_set) return fail(QED3_ERR_STATE, "call qed3_dirac_ext_set_links first");
  const int Ns = e->d2->Ns;
  if (s < 0 || s >= e->Nt || ix < 0 || ix >= Ns || a < 0 || a > 1)
    return fail(QED3_ERR_ARG, "source point out of range");
  const long long nd = 4LL * Ns * e->Nt;
  double* buf = nullptr;
  if (cudaMalloc(&buf, size_t(nd) * 2 * sizeof(double)) != cudaSuccess) return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  double *src1 = buf, *src = buf + nd;
  auto body = [&]() -> int {
    const double one = 1.0;
    QED3_CUDA_TRY(cudaMemsetAsync(src1, 0, nd * sizeof(double), st));
    QED3_CUDA_TRY(cudaMemcpyAsync(src1 + 2 * ((size_t(s) * Ns + ix) * 2 + a), &one, sizeof(double),
                                  cudaMemcpyHostToDevice, st));
    int rc = ext_apply(e, dagger ? QED3_OP_D : QED3_OP_DDAG, src, src1, st);
    if (rc) return rc;
    qed3_solve_report r{};
    rc = ext_cg(e, sink, src, prm, &r, st, dagger ? QED3_OP_DDDAG : QED3_OP_DDAGD);
    if (rep) *rep = r;
    if (!rc && r.status != QED3_OK) rc = fail(QED3_ERR_NOCONV, "propagator solve did not converge");
    return rc;
  };
  const int rc = body();
  cudaStreamSynchronize(st);
  cudaFree(buf);
  return rc;
}

}  // namespace qed3
