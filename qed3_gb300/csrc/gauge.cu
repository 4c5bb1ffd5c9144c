// Gauge side and forces on the device (sm_103a).
//
//  * plaquette angles theta_f = sum of oriented link angles around each dual
//    face (U1onS2::plaquette_angle, src/dual/gauge.h:90-102)
//  * Wilson action with area weights w_f = mean_vol / vol_f
//    (src/both/action.h:21-30): compact -beta sum w cos(theta),
//    non-compact beta/2 sum w theta^2
//  * gauge force per link from its two faces (src/both/action.h:32-48);
//    compact force exact (sin theta) or the reference's (theta,
//    src/dual/action.h:37)
//  * Wilson fermion force for ALL links in one kernel, F_l = -2 Re <D eta,
//    dD/dA_l eta> (DiracPf::grad_deviceAsyncLaunch, src/both_3d/dirac_pf.h:107-122,
//    which launched a full-lattice SpMV per link: O(N_l N) -> O(N_l) here)
//  * pure-gauge HMC leapfrog (HMCPureGauge, src/both_3d/hmc.h:212-296) with
//    dH accumulated as per-term differences in FP64.

#include <cmath>
#include <cstdint>
#include <fstream>
#include <functional>
#include <sstream>
#include <string>
#include <random>
#include <vector>

#include "device.cuh"
#include "batched_impl.h"
#include "blas_impl.h"
#include "dirac_impl.h"
#include "gauge_impl.h"
#include "handles.h"
#include "overlap_impl.h"

namespace qed3 {

static inline int nblk(long long n, int t = 256) { return int((n + t - 1) / t); }

__global__ void k_plaquettes(int Nf, const int32_t* __restrict__ off, const int32_t* __restrict__ flink,
                             const int8_t* __restrict__ fsign, const double* __restrict__ A, double* __restrict__ th) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= Nf) return;
  double s = 0.0;
  for (int e = off[f]; e < off[f + 1]; e++) s += double(fsign[e]) * A[flink[e]];
  th[f] = s;
}

__device__ __forceinline__ double face_energy(double th, int compact) {
  return compact ? -cos(th) : 0.5 * th * th;
}
__device__ __forceinline__ double face_grad(double th, int compact, int exact) {
  return (compact && exact) ? sin(th) : th;
}

// Block partial sums of one or two per-element quantities (deterministic:
// the host adds the block partials in order).
template <class F>
__global__ void k_sum(int n, F f, double* __restrict__ part) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += f(i);
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

struct ActionTerm {
  const double* th;
  const double* w;
  int compact;
  __device__ double operator()(int f) const { return w[f] * face_energy(th[f], compact); }
};
struct ActionDiff {  // w (e(theta1) - e(theta0))
  const double* th1;
  const double* th0;
  const double* w;
  int compact;
  __device__ double operator()(int f) const {
    if (compact) {
      // -cos a + cos b = 2 sin((a+b)/2) sin((a-b)/2): no cancellation
      const double a = th1[f], b = th0[f];
      return w[f] * 2.0 * sin(0.5 * (a + b)) * sin(0.5 * (a - b));
    }
    return w[f] * 0.5 * (th1[f] - th0[f]) * (th1[f] + th0[f]);
  }
};
struct KinDiff {  // (pi1^2 - pi0^2)/2
  const double* p1;
  const double* p0;
  __device__ double operator()(int l) const { return 0.5 * (p1[l] - p0[l]) * (p1[l] + p0[l]); }
};
struct Kin {
  const double* p;
  __device__ double operator()(int l) const { return 0.5 * p[l] * p[l]; }
};
struct CosTerm {
  const double* th;
  __device__ double operator()(int f) const { return cos(th[f]); }
};

// Each dual link borders exactly two dual faces.
__global__ void k_gauge_force(int Nl, const int32_t* __restrict__ lf, const int8_t* __restrict__ ls,
                              const double* __restrict__ th, const double* __restrict__ w, double beta, int compact,
                              int exact, double* __restrict__ F) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Nl) return;
  const int f0 = lf[2 * l], f1 = lf[2 * l + 1];
  F[l] = beta * (w[f0] * face_grad(th[f0], compact, exact) * double(ls[2 * l]) +
                 w[f1] * face_grad(th[f1], compact, exact) * double(ls[2 * l + 1]));
}

__global__ void k_axpy(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

// F_l = -2 Re[ (D eta)_x^dag (i H_xy eta_y) + (D eta)_y^dag (-i H_yx eta_x) ]
// with D eta and eta in internal order.
__global__ void k_fermion_force(int Nl, int Ns, const int32_t* __restrict__ lx, const int32_t* __restrict__ ly,
                                const int8_t* __restrict__ kx, const int8_t* __restrict__ ky, const M64* __restrict__ H,
                                const S64* __restrict__ eta, const S64* __restrict__ deta, double* __restrict__ F) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Nl) return;
  const int x = lx[l], y = ly[l];
  const M64 hxy = H[size_t(kx[l]) * Ns + x], hyx = H[size_t(ky[l]) * Ns + y];
  const Sp64 ex = ld64(eta, x), ey = ld64(eta, y), dx = ld64(deta, x), dy = ld64(deta, y);
  // u = H_xy eta_y, v = H_yx eta_x
  const double2 u0 = cfma(hxy.h01, ey.s1, cmul(hxy.h00, ey.s0));
  const double2 u1 = cfma(hxy.h11, ey.s1, cmul(hxy.h10, ey.s0));
  const double2 v0 = cfma(hyx.h01, ex.s1, cmul(hyx.h00, ex.s0));
  const double2 v1 = cfma(hyx.h11, ex.s1, cmul(hyx.h10, ex.s0));
  // Re[conj(a) * (i b)] = -(a.x b.y - a.y b.x) = a.y b.x - a.x b.y
  auto re_ci = [](double2 a, double2 b) { return a.y * b.x - a.x * b.y; };
  const double inner = re_ci(dx.s0, u0) + re_ci(dx.s1, u1) - re_ci(dy.s0, v0) - re_ci(dy.s1, v1);
  F[l] = -2.0 * inner;
}

// Re <u, (dD/dA_l) v> over the two blocks of link l = (x, y):
//   conj(u_x) (i H_xy v_y) + conj(u_y) (-i H_yx v_x)
__device__ __forceinline__ double link_inner(const M64& hxy, const M64& hyx, const Sp64& ux, const Sp64& uy,
                                             const Sp64& vx, const Sp64& vy) {
  const double2 a0 = cfma(hxy.h01, vy.s1, cmul(hxy.h00, vy.s0));
  const double2 a1 = cfma(hxy.h11, vy.s1, cmul(hxy.h10, vy.s0));
  const double2 b0 = cfma(hyx.h01, vx.s1, cmul(hyx.h00, vx.s0));
  const double2 b1 = cfma(hyx.h11, vx.s1, cmul(hyx.h10, vx.s0));
  // Re[conj(a) (i b)] = a.y b.x - a.x b.y
  auto re_ci = [](double2 a, double2 b) { return a.y * b.x - a.x * b.y; };
  return re_ci(ux.s0, a0) + re_ci(ux.s1, a1) - re_ci(uy.s0, b0) - re_ci(uy.s1, b1);
}

// Overlap force over all links (internal-order fields, np poles back to back):
//   F_l = sum_m c_m (Re<DZ_m, dD Y_m> + Re<DY_m, dD Z_m>) + c_w Re<eta, dD w>
struct OvForceCoef {
  double c[64];
  double cw;
  int np;
};
__global__ void k_overlap_force(int Nl, int Ns, const int32_t* __restrict__ lx, const int32_t* __restrict__ ly,
                                const int8_t* __restrict__ kx, const int8_t* __restrict__ ky,
                                const M64* __restrict__ H, const S64* __restrict__ Z, const S64* __restrict__ Y,
                                const S64* __restrict__ DZ, const S64* __restrict__ DY, const S64* __restrict__ eta,
                                const S64* __restrict__ w, OvForceCoef co, double* __restrict__ F) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Nl) return;
  const int x = lx[l], y = ly[l];
  const M64 hxy = H[size_t(kx[l]) * Ns + x], hyx = H[size_t(ky[l]) * Ns + y];
  double f = co.cw * link_inner(hxy, hyx, ld64(eta, x), ld64(eta, y), ld64(w, x), ld64(w, y));
  for (int m = 0; m < co.np; m++) {
    const size_t o = size_t(m) * Ns;
    const double t = link_inner(hxy, hyx, ld64(DZ + o, x), ld64(DZ + o, y), ld64(Y + o, x), ld64(Y + o, y)) +
                     link_inner(hxy, hyx, ld64(DY + o, x), ld64(DY + o, y), ld64(Z + o, x), ld64(Z + o, y));
    f += co.c[m] * t;
  }
  F[l] = f;
}

int overlap_force_links(qed3_dirac_s* d, int np, const double* c, double cw, const S64* Z, const S64* Y,
                        const S64* DZ, const S64* DY, const S64* eta, const S64* w, double* F, cudaStream_t st) {
  if (np > 64) return fail(QED3_ERR_ARG, "at most 64 poles");
  const DeviceLattice& D = d->lat->dev;
  OvForceCoef co{};
  for (int m = 0; m < np; m++) co.c[m] = c[m];
  co.cw = cw;
  co.np = np;
  k_overlap_force<<<nblk(D.Nl), 256, 0, st>>>(D.Nl, d->Ns, D.link_x, D.link_y, D.link_kx, D.link_ky, d->H, Z, Y, DZ,
                                              DY, eta, w, co, F);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int gauge_prepare(qed3_lattice_s* lat) {
  GaugeDev& G = lat->gauge;
  if (G.ready) return QED3_OK;
  if (!lat->dev.nbr) {
    int rc = lattice_upload(lat);
    if (rc) return rc;
  }
  const HostLattice& L = lat->host;
  const int Nl = L.n_links, Nf = L.n_faces;
  std::vector<int32_t> lf(size_t(2) * Nl, -1);
  std::vector<int8_t> ls(size_t(2) * Nl, 0);
  std::vector<int> cnt(Nl, 0);
  for (int f = 0; f < Nf; f++)
    for (int e = L.face_offsets[f]; e < L.face_offsets[f + 1]; e++) {
      const int l = L.face_links[e];
      if (cnt[l] >= 2) return fail(QED3_ERR_STATE, "link in more than two faces");
      lf[2 * l + cnt[l]] = f;
      ls[2 * l + cnt[l]] = L.face_link_sign[e];
      cnt[l]++;
    }
  for (int l = 0; l < Nl; l++)
    if (cnt[l] != 2) return fail(QED3_ERR_STATE, "link not in two faces");
  QED3_CUDA_TRY(cudaMalloc(&G.link_face, lf.size() * sizeof(int32_t)));
  QED3_CUDA_TRY(cudaMalloc(&G.link_fsign, ls.size() * sizeof(int8_t)));
  QED3_CUDA_TRY(cudaMemcpy(G.link_face, lf.data(), lf.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMemcpy(G.link_fsign, ls.data(), ls.size() * sizeof(int8_t), cudaMemcpyHostToDevice));
  QED3_CUDA_TRY(cudaMalloc(&G.th0, size_t(Nf) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.th1, size_t(Nf) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.pi, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.pi0, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.F, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.A0, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&G.part, 1024 * sizeof(double)));
  G.ready = true;
  return QED3_OK;
}

void gauge_free(qed3_lattice_s* lat) {
  GaugeDev& G = lat->gauge;
  void* ptrs[] = {G.link_face, G.link_fsign, G.th0, G.th1, G.pi, G.pi0, G.F, G.A0, G.part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  G = GaugeDev{};
}

template <class F>
static int reduce(int n, F f, double* part, double* out, cudaStream_t st) {
  const int g = std::min(1024, std::max(1, nblk(n)));
  k_sum<<<g, 256, 0, st>>>(n, f, part);
  QED3_CUDA_TRY(cudaGetLastError());
  std::vector<double> h(g);
  QED3_CUDA_TRY(cudaMemcpyAsync(h.data(), part, size_t(g) * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s;
  return QED3_OK;
}

int gauge_plaquettes(qed3_lattice_s* lat, const double* A, double* th, cudaStream_t st) {
  const DeviceLattice& D = lat->dev;
  k_plaquettes<<<nblk(D.Nf), 256, 0, st>>>(D.Nf, D.face_off, D.face_link, D.face_sign, A, th);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int gauge_plaquette_avg(qed3_lattice_s* lat, const double* A, double* theta, double* avg, cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  double* th = theta ? theta : lat->gauge.th0;
  if ((rc = gauge_plaquettes(lat, A, th, st))) return rc;
  if (avg) {
    double s;
    if ((rc = reduce(lat->dev.Nf, CosTerm{th}, lat->gauge.part, &s, st))) return rc;
    *avg = s / lat->dev.Nf;  // U1onS2::average_plaquette, src/dual/gauge.h:104-110
  }
  return QED3_OK;
}

int gauge_action(qed3_lattice_s* lat, const double* A, double beta, int compact, double* S, cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  if ((rc = gauge_plaquettes(lat, A, lat->gauge.th0, st))) return rc;
  double s;
  if ((rc = reduce(lat->dev.Nf, ActionTerm{lat->gauge.th0, lat->dev.face_weight, compact}, lat->gauge.part, &s, st)))
    return rc;
  *S = beta * s;
  return QED3_OK;
}

int gauge_force(qed3_lattice_s* lat, const double* A, double beta, int compact, int exact, double* F, cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  const DeviceLattice& D = lat->dev;
  if ((rc = gauge_plaquettes(lat, A, lat->gauge.th1, st))) return rc;
  k_gauge_force<<<nblk(D.Nl), 256, 0, st>>>(D.Nl, lat->gauge.link_face, lat->gauge.link_fsign, lat->gauge.th1,
                                            D.face_weight, beta, compact, exact, F);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

int fermion_force(qed3_dirac_s* d, const double* eta_ref, double* F, cudaStream_t st) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  const DeviceLattice& D = d->lat->dev;
  int rc = field_import(d, QED3_PREC_F64, d->tmp_in, eta_ref, 1, st);
  if (rc) return rc;
  if ((rc = dirac_apply_field(d, QED3_OP_D, QED3_PREC_F64, d->tmp_out, d->tmp_in, 1, st))) return rc;
  k_fermion_force<<<nblk(D.Nl), 256, 0, st>>>(D.Nl, d->Ns, D.link_x, D.link_y, D.link_kx, D.link_ky, d->H, d->tmp_in,
                                              d->tmp_out, F);
  QED3_CUDA_TRY(cudaGetLastError());
  return QED3_OK;
}

// ---- RNG: ParallelRng2 (src/both/rng.h:76-125) ------------------------------------
struct RngEngine {
  std::mt19937_64 mt;
  std::normal_distribution<double> g;
  std::uniform_real_distribution<double> u;
  std::uniform_int_distribution<int> z2{1, 2};  // SingleRng::dist_z2(1,2)
};
struct HostRng {
  RngEngine master;
  std::vector<RngEngine> links, sites;
};

}  // namespace qed3

struct qed3_rng_s {
  qed3::HostRng r;
};

namespace qed3 {

// The reference seeds every engine through SingleRng::reseed(const int): the
// master's 64-bit draw is narrowed to a signed 32-bit int and that int is
// widened again (sign-extended) by mt19937_64::seed.
static inline std::uint64_t engine_seed(std::uint64_t draw) {
  return std::uint64_t(std::int64_t(std::int32_t(std::uint32_t(draw & 0xffffffffu))));
}

qed3_rng_s* rng_create(int n_links, int n_sites, int seed) {
  auto* r = new qed3_rng_s;
  r->r.links.resize(n_links);
  r->r.sites.resize(n_sites);
  r->r.master.mt.seed(engine_seed(std::uint64_t(std::int64_t(seed))));
  for (auto& e : r->r.links) e.mt.seed(engine_seed(r->r.master.mt()));
  for (auto& e : r->r.sites) e.mt.seed(engine_seed(r->r.master.mt()));
  return r;
}
void rng_destroy(qed3_rng_s* r) { delete r; }

// Checkpoint in the layout of ParallelRngExt::ckpoint / read
// (src/both_3d/rng.h:131-168, Nt = 1): the master engine, then every link
// engine, then every site engine, each as SingleRng's operator<< writes it
// (src/both_3d/rng.h:23-30): four lines -- the mt19937_64 state, then the
// normal, uniform-real and uniform-int distribution states, in the standard
// library's stream format.
int rng_save(const qed3_rng_s* r, const char* path) {
  std::ofstream os(path);
  if (!os) return fail(QED3_ERR_ARG, std::string("cannot write ") + path);
  auto put = [&](const RngEngine& e) {
    os << e.mt << std::endl;
    os << e.g << std::endl;
    os << e.u << std::endl;
    os << e.z2 << std::endl;
  };
  put(r->r.master);
  for (const auto& e : r->r.links) put(e);
  for (const auto& e : r->r.sites) put(e);
  if (!os) return fail(QED3_ERR_ARG, std::string("write failed: ") + path);
  return QED3_OK;
}

int rng_load(qed3_rng_s* r, const char* path) {
  std::ifstream is(path);
  if (!is) return fail(QED3_ERR_ARG, std::string("cannot read ") + path);
  HostRng tmp;
  tmp.links.resize(r->r.links.size());
  tmp.sites.resize(r->r.sites.size());
  auto get = [&](RngEngine& e) -> bool {
    std::string line;
    std::istringstream ss;
    if (!std::getline(is, line)) return false;
    ss.str(line);
    if (!(ss >> e.mt)) return false;
    if (!std::getline(is, line)) return false;
    ss.clear();
    ss.str(line);
    if (!(ss >> e.g)) return false;
    if (!std::getline(is, line)) return false;
    ss.clear();
    ss.str(line);
    if (!(ss >> e.u)) return false;
    if (!std::getline(is, line)) return false;
    ss.clear();
    ss.str(line);
    return bool(ss >> e.z2);
  };
  bool ok = get(tmp.master);
  for (auto& e : tmp.links) ok = ok && get(e);
  for (auto& e : tmp.sites) ok = ok && get(e);
  if (!ok) return fail(QED3_ERR_ARG, std::string("not a random-stream checkpoint of this size: ") + path);
  r->r = std::move(tmp);
  return QED3_OK;
}
void rng_gaussian_links(qed3_rng_s* r, double width, double* out) {
  for (size_t l = 0; l < r->r.links.size(); l++) out[l] = width * r->r.links[l].g(r->r.links[l].mt);
}
// GaugeExt::gaussian's temporal part (src/both_3d/gauge_ext.h:145-149): one
// Gaussian per site engine, in engine order
void rng_counts(const qed3_rng_s* r, size_t* n_links, size_t* n_sites) {
  *n_links = r->r.links.size();
  *n_sites = r->r.sites.size();
}

void rng_gaussian_sites(qed3_rng_s* r, double width, double* out) {
  for (size_t x = 0; x < r->r.sites.size(); x++) out[x] = width * r->r.sites[x].g(r->r.sites[x].mt);
}
void rng_gaussian_spinor(qed3_rng_s* r, double* out) {
  // ParallelRngExt::fill_gaussian, src/both_3d/rng.h:122-129
  for (size_t x = 0; x < r->r.sites.size(); x++)
    for (int a = 0; a < 2; a++) {
      auto& e = r->r.sites[x];
      const double re = e.g(e.mt);
      const double im = e.g(e.mt);
      out[4 * x + 2 * a] = re / std::sqrt(2.0);
      out[4 * x + 2 * a + 1] = im / std::sqrt(2.0);
    }
}
double rng_uniform(qed3_rng_s* r) { return r->r.master.u(r->r.master.mt); }
void rng_z2_spinor(qed3_rng_s* r, double* out) {
  // FermionVector::set_random, src/dual/valence.h:54-60 (z2_site draws 1 or 2)
  const double nrm = std::sqrt(2.0 * double(r->r.sites.size()));
  for (size_t x = 0; x < r->r.sites.size(); x++)
    for (int a = 0; a < 2; a++) {
      auto& e = r->r.sites[x];
      const double re = e.z2(e.mt);
      const double im = e.z2(e.mt);
      out[4 * x + 2 * a] = re / nrm;
      out[4 * x + 2 * a + 1] = im / nrm;
    }
}

int hmc_pure_gauge(qed3_lattice_s* lat, qed3_rng_s* rng, double* A, double beta, int compact, int exact, double tmax,
                   int nsteps, int no_reject, int* accepted, double* dH_out, cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  GaugeDev& G = lat->gauge;
  const DeviceLattice& D = lat->dev;
  const int Nl = D.Nl, Nf = D.Nf;
  std::vector<double> pi(Nl);
  rng_gaussian_links(rng, 1.0, pi.data());
  QED3_CUDA_TRY(cudaMemcpyAsync(G.pi, pi.data(), size_t(Nl) * sizeof(double), cudaMemcpyHostToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(G.pi0, G.pi, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(G.A0, A, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if ((rc = gauge_plaquettes(lat, A, G.th0, st))) return rc;  // theta at the start
  const double tau = tmax / nsteps;
  for (int n = 0; n < nsteps; n++) {
    if ((rc = gauge_force(lat, A, beta, compact, exact, G.F, st))) return rc;
    k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, -0.5 * tau, G.F, G.pi);
    k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, tau, G.pi, A);
    if ((rc = gauge_force(lat, A, beta, compact, exact, G.F, st))) return rc;
    k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, -0.5 * tau, G.F, G.pi);
  }
  QED3_CUDA_TRY(cudaGetLastError());
  if ((rc = gauge_plaquettes(lat, A, G.th1, st))) return rc;
  double dk, ds;
  if ((rc = reduce(Nl, KinDiff{G.pi, G.pi0}, G.part, &dk, st))) return rc;
  if ((rc = reduce(Nf, ActionDiff{G.th1, G.th0, D.face_weight, compact}, G.part, &ds, st))) return rc;
  const double dH = dk + beta * ds;
  *dH_out = dH;
  const double r = std::min(1.0, std::exp(-dH));
  const double a = rng_uniform(rng);
  if (a < r || no_reject) {
    *accepted = 1;
  } else {
    *accepted = 0;
    QED3_CUDA_TRY(cudaMemcpyAsync(A, G.A0, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  return QED3_OK;
}


// The fermion side of a trajectory: set the operator from the links,
// phi = D^dag xi, eta = (D^dag D)^{-1} phi, and the force
// F_l = dS/dA_l = -2 Re <eta, d(D) eta>-type term of the operator.
struct HmcFermion {
  std::function<int(const double* A)> update;
  std::function<int(double* phi, const double* xi)> apply_dag;
  std::function<int(double* eta, const double* phi, int* iters)> solve;
  // optional: every pseudofermion's solve at once (eta, phi: npf fields back to back)
  std::function<int(double* eta, const double* phi, int npf, int* iters)> solve_all;
  std::function<int(const double* eta, double* F)> force;
};

// HMC::run (npf = 1) / HMC2::run (src/both_3d/hmc.h:75-110, :172-200), every
// field on the device: momenta and one xi per pseudofermion from the RNG
// streams (fill_gaussian order), phi = D^dag xi, eta = (D^dag D)^{-1} phi;
// H = |pi|^2/2 + S_g + sum Re<phi, eta>, dH formed term by term; Metropolis
// with the master engine's uniform; links and operator restored on rejection.
// Integrators:
//  * QED3_INTEGRATOR_LEAPFROG_ML, ExplicitLeapfrogML
//    (src/both_3d/integrator.h:58-168): half fermion kick per pseudofermion;
//    nsteps of [gauge leapfrog with nsteps_inner steps of tau/nsteps_inner,
//    operator update, per pseudofermion: solve + kick (half on the last)];
//  * QED3_INTEGRATOR_LEAPFROG, ExplicitLeapfrog (src/dual/integrator.h:9-53):
//    nsteps of [pi -= tau/2 (F_g + F_f), U += tau pi, operator update and
//    solves, pi -= tau/2 (F_g + F_f)] (F_f summed over the pseudofermions).
static int hmc_trajectory(qed3_lattice_s* lat, const HmcFermion& fo, long long nd, qed3_rng_s* rng, double* A,
                          double beta, int compact, int exact, double tmax, int nsteps, int nsteps_inner, int npf,
                          int integrator, int no_reject, int* accepted, double* dH_out, int* cg_iters,
                          cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  GaugeDev& G = lat->gauge;
  const DeviceLattice& D = lat->dev;
  const int Nl = D.Nl, Nf = D.Nf;
  std::vector<double> pi(Nl), xi(nd * npf);
  rng_gaussian_links(rng, 1.0, pi.data());
  for (int k = 0; k < npf; k++) rng_gaussian_spinor(rng, xi.data() + nd * k);
  double *phi = nullptr, *eta = nullptr, *eta0 = nullptr, *dxi = nullptr, *Ff = nullptr, *part = nullptr;
  auto cleanup = [&]() {
    for (double* p : {phi, eta, eta0, dxi, Ff, part})
      if (p) cudaFree(p);
  };
  const size_t vbytes = size_t(nd) * npf * sizeof(double);
  if (cudaMalloc(&phi, vbytes) != cudaSuccess || cudaMalloc(&eta, vbytes) != cudaSuccess ||
      cudaMalloc(&eta0, vbytes) != cudaSuccess || cudaMalloc(&dxi, vbytes) != cudaSuccess ||
      cudaMalloc(&Ff, size_t(Nl) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&part, 4096 * sizeof(double)) != cudaSuccess) {
    cleanup();
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  int its = 0;
  auto solve_eta = [&](int k) -> int { return fo.solve(eta + nd * k, phi + nd * k, &its); };
  // the npf solves of one operator update: one batched launch when available
  // (their order does not matter: no solve depends on the momenta)
  auto solve_all = [&]() -> int {
    if (fo.solve_all && npf > 1) return fo.solve_all(eta, phi, npf, &its);
    for (int k = 0; k < npf; k++)
      if (int e = solve_eta(k)) return e;
    return QED3_OK;
  };
  auto run = [&]() -> int {
    int e;
    QED3_CUDA_TRY(cudaMemcpyAsync(G.pi, pi.data(), size_t(Nl) * sizeof(double), cudaMemcpyHostToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(G.pi0, G.pi, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(G.A0, A, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
    QED3_CUDA_TRY(cudaMemcpyAsync(dxi, xi.data(), vbytes, cudaMemcpyHostToDevice, st));
    if ((e = fo.update(A))) return e;
    for (int k = 0; k < npf; k++)
      if ((e = fo.apply_dag(phi + nd * k, dxi + nd * k))) return e;
    if ((e = solve_all())) return e;
    QED3_CUDA_TRY(cudaMemcpyAsync(eta0, eta, vbytes, cudaMemcpyDeviceToDevice, st));
    if ((e = gauge_plaquettes(lat, A, G.th0, st))) return e;
    const double tau = tmax / nsteps, tau_in = tau / nsteps_inner;
    auto fermion_kick = [&](int k, double c) -> int {
      int f = fo.force(eta + nd * k, Ff);
      if (!f) k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, -c, Ff, G.pi);
      return f;
    };
    auto gauge_kick = [&](double c) -> int {
      int f = gauge_force(lat, A, beta, compact, exact, G.F, st);
      if (!f) k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, -c, G.F, G.pi);
      return f;
    };
    // pi -= c (F_g + sum_k F_f,k): the forces summed first, as (dSg + dSf)
    auto full_kick = [&](double c) -> int {
      int f = gauge_force(lat, A, beta, compact, exact, G.F, st);
      for (int k = 0; k < npf && !f; k++) {
        f = fo.force(eta + nd * k, Ff);
        if (!f) k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, 1.0, Ff, G.F);
      }
      if (!f) k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, -c, G.F, G.pi);
      return f;
    };
    if (integrator == QED3_INTEGRATOR_LEAPFROG) {
      for (int n = 0; n < nsteps; n++) {
        if ((e = full_kick(0.5 * tau))) return e;
        k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, tau, G.pi, A);
        if ((e = fo.update(A))) return e;
        if ((e = solve_all())) return e;
        if ((e = full_kick(0.5 * tau))) return e;
      }
    }
    for (int k = 0; k < npf && integrator != QED3_INTEGRATOR_LEAPFROG; k++)
      if ((e = fermion_kick(k, 0.5 * tau))) return e;
    for (int n = 0; n < nsteps && integrator != QED3_INTEGRATOR_LEAPFROG; n++) {
      if ((e = gauge_kick(0.5 * tau_in))) return e;
      for (int m = 0; m < nsteps_inner; m++) {
        k_axpy<<<nblk(Nl), 256, 0, st>>>(Nl, tau_in, G.pi, A);
        if ((e = gauge_kick((m != nsteps_inner - 1 ? 1.0 : 0.5) * tau_in))) return e;
      }
      if ((e = fo.update(A))) return e;
      if ((e = solve_all())) return e;
      for (int k = 0; k < npf; k++)
        if ((e = fermion_kick(k, (n != nsteps - 1 ? 1.0 : 0.5) * tau))) return e;
    }
    QED3_CUDA_TRY(cudaGetLastError());
    if ((e = gauge_plaquettes(lat, A, G.th1, st))) return e;
    double dk, ds, dsf = 0;
    if ((e = reduce(Nl, KinDiff{G.pi, G.pi0}, G.part, &dk, st))) return e;
    if ((e = reduce(Nf, ActionDiff{G.th1, G.th0, D.face_weight, compact}, G.part, &ds, st))) return e;
    for (int k = 0; k < npf; k++) {
      double sf0, sf1;
      if ((e = vec_zdot(nd / 2, phi + nd * k, eta + nd * k, part, &sf1, nullptr, st))) return e;
      if ((e = vec_zdot(nd / 2, phi + nd * k, eta0 + nd * k, part, &sf0, nullptr, st))) return e;
      dsf += sf1 - sf0;
    }
    const double dH = dk + beta * ds + dsf;
    *dH_out = dH;
    if (cg_iters) *cg_iters = its;
    const double r = std::min(1.0, std::exp(-dH));
    const double a = rng_uniform(rng);
    if (a < r || no_reject) {
      *accepted = 1;
    } else {
      *accepted = 0;
      QED3_CUDA_TRY(cudaMemcpyAsync(A, G.A0, size_t(Nl) * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if ((e = fo.update(A))) return e;
    }
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
    return QED3_OK;
  };
  rc = run();
  cleanup();
  return rc;
}

int hmc_fermion(qed3_lattice_s* lat, qed3_dirac_s* d, qed3_rng_s* rng, double* A, double beta, int compact, int exact,
                double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double tol, int prec, int no_reject,
                int* accepted, double* dH_out, int* cg_iters, cudaStream_t st) {
  const qed3_solve_params sp{tol, 0, prec, 0.1, 0.0, 0};
  HmcFermion fo;
  fo.update = [&](const double* U) { return dirac_set_links(d, U, 1, st); };
  fo.apply_dag = [&](double* phi, const double* xi) { return dirac_apply_ref(d, QED3_OP_DDAG, phi, xi, st); };
  fo.solve = [&](double* eta, const double* phi, int* its) {
    qed3_solve_report r{};
    int e = cg_solve(d, eta, phi, &sp, &r, st);
    *its += r.iters;
    if (!e && r.status != QED3_OK) e = fail(QED3_ERR_NOCONV, "pseudofermion solve did not converge");
    return e;
  };
  fo.force = [&](const double* eta, double* F) { return fermion_force(d, eta, F, st); };
  // several pseudofermions of the one operator: one batched persistent launch
  // per operator update, the right-hand sides in one tile
  qed3_batch_s* bt = nullptr;
  fo.solve_all = [&](double* eta, const double* phi, int n, int* its) -> int {
    if (!bt) {
      const int tile = n <= 1 ? 1 : n <= 2 ? 2 : n <= 4 ? 4 : 8;
      qed3_dirac_s* ops[1] = {d};
      const int nr[1] = {n};
      if (int e = batch_create(1, ops, nr, prec, tile, 128, &bt)) return e;
    }
    double* xs[1] = {eta};
    const double* bs[1] = {phi};
    std::vector<qed3_solve_report> reps(static_cast<size_t>(n));
    int e = batch_solve(bt, xs, bs, nullptr, &sp, reps.data(), nullptr, st);
    for (const auto& r : reps) {
      *its += r.iters;
      if (!e && r.status != QED3_OK) e = fail(QED3_ERR_NOCONV, "pseudofermion solve did not converge");
    }
    return e;
  };
  const int rc = hmc_trajectory(lat, fo, 4LL * d->Ns, rng, A, beta, compact, exact, tmax, nsteps, nsteps_inner, npf,
                                integrator, no_reject, accepted, dH_out, cg_iters, st);
  if (bt) batch_destroy(bt);
  return rc;
}

// Overlap fermions (the reference's IS_OVERLAP build of HMC2): the operator
// update is Overlap::update (src/both_3d/overlap.h:207-216: Wilson links, then
// lambda bounds by power iterations and new Zolotarev coefficients) unless
// fixed bounds lmin, lmax > 0 are given; eta = (D_ov^dag D_ov)^{-1} phi by the
// outer CG; the force is the overlap force (src/both_3d/overlap.h:393-470).
int hmc_overlap(qed3_lattice_s* lat, qed3_overlap_s* ov, qed3_rng_s* rng, double* A, double beta, int compact,
                int exact, double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double lmin, double lmax,
                double tol, double tol_inner, int no_reject, int* accepted, double* dH_out, int* cg_iters,
                cudaStream_t st) {
  qed3_dirac_s* d = overlap_dirac(ov);
  HmcFermion fo;
  fo.update = [&](const double* U) {
    int e = dirac_set_links(d, U, 1, st);
    return e ? e : overlap_update(ov, lmin, lmax, tol_inner, st);
  };
  fo.apply_dag = [&](double* phi, const double* xi) {
    return overlap_apply(ov, QED3_OP_DDAG, phi, xi, tol_inner, nullptr, st);
  };
  fo.solve = [&](double* eta, const double* phi, int* its) {
    qed3_solve_report r{};
    int e = overlap_solve(ov, eta, phi, tol, tol_inner, 100000, 0, &r, st);
    *its += r.iters;
    if (!e && r.status != QED3_OK) e = fail(QED3_ERR_NOCONV, "overlap pseudofermion solve did not converge");
    return e;
  };
  fo.force = [&](const double* eta, double* F) { return overlap_force(ov, eta, F, tol_inner, nullptr, st); };
  return hmc_trajectory(lat, fo, 4LL * d->Ns, rng, A, beta, compact, exact, tmax, nsteps, nsteps_inner, npf,
                        integrator, no_reject, accepted, dH_out, cg_iters, st);
}

}  // namespace qed3

// ===========================================================================
// S^2 x S^1 gauge side: U1WilsonExt (src/both_3d/action_ext.h:4-161) and the
// Polyakov loop (src/both_3d/obs.h:4-10).  Links A[Nt][Nl] spatial, then
// A[Nt][Ns] temporal (reference site order).  Plaquettes:
//   spatial  theta_s(s, f) = sum of the face's oriented slice-s links,
//   temporal theta_t(s, l) = A_s[l] + A_t(s, y) - A_{s+1}[l] - A_t(s, x), l = (x, y);
// action sum_s [sum_f beta_s[f] theta_s^2 / 2 + sum_l beta_t[l] theta_t^2 / 2]
// with beta_s = at / vols[f] / gsq, beta_t = 2 / at * link_volume / ell^2 / gsq.
// ===========================================================================
namespace qed3 {

__global__ void k_ext_plaq(int Nt, int Nl, int Ns, int Nf, const int32_t* __restrict__ off,
                           const int32_t* __restrict__ flink, const int8_t* __restrict__ fsign,
                           const int32_t* __restrict__ lx, const int32_t* __restrict__ ly,
                           const int32_t* __restrict__ perm, const double* __restrict__ A, double* __restrict__ ths,
                           double* __restrict__ tht) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nsp = (long long)Nt * Nf;
  if (idx < nsp) {
    const int s = int(idx / Nf), f = int(idx % Nf);
    const double* As = A + size_t(s) * Nl;
    double t = 0.0;
    for (int e = off[f]; e < off[f + 1]; e++) t += double(fsign[e]) * As[flink[e]];
    ths[idx] = t;
  } else if (idx < nsp + (long long)Nt * Nl) {
    const long long j = idx - nsp;
    const int s = int(j / Nl), l = int(j % Nl), s1 = (s + 1) % Nt;
    const double* At = A + size_t(Nt) * Nl + size_t(s) * Ns;
    const int x = perm[lx[l]], y = perm[ly[l]];
    double t = 0.0;
    t += A[size_t(s) * Nl + l];
    t += At[y];
    t -= A[size_t(s1) * Nl + l];
    t -= At[x];
    tht[j] = t;
  }
}

struct ExtAction {
  const double *ths, *tht, *bs, *bt;
  long long nsp;
  int Nf, Nl;
  __device__ double operator()(int i) const {
    if (i < nsp) return 0.5 * bs[i % Nf] * ths[i] * ths[i];
    const long long j = i - nsp;
    return 0.5 * bt[j % Nl] * tht[j] * tht[j];
  }
};

// spatial force per (s, l): its two faces (ascending face index), then the
// temporal plaquettes of slices s and s-1, in the reference's order of updates
__global__ void k_ext_force_s(int Nt, int Nl, int Nf, const int32_t* __restrict__ lf, const int8_t* __restrict__ ls,
                              const double* __restrict__ ths, const double* __restrict__ tht,
                              const double* __restrict__ bs, const double* __restrict__ bt, double* __restrict__ F) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Nt * Nl) return;
  const int s = int(idx / Nl), l = int(idx % Nl), sm = (s + Nt - 1) % Nt;
  const int f0 = lf[2 * l], f1 = lf[2 * l + 1];
  double v = 0.0;
  v += bs[f0] * ths[size_t(s) * Nf + f0] * double(ls[2 * l]);
  v += bs[f1] * ths[size_t(s) * Nf + f1] * double(ls[2 * l + 1]);
  v += bt[l] * tht[size_t(s) * Nl + l];
  v -= bt[l] * tht[size_t(sm) * Nl + l];
  F[idx] = v;
}

// temporal force per (s, x): the three incident links in increasing link
// index (the reference's loop order), +grad at the link's end, -grad at its start
__global__ void k_ext_force_t(int Nt, int Nl, int Ns, const int32_t* __restrict__ hop_link,
                              const int8_t* __restrict__ hop_sign, const int32_t* __restrict__ perm,
                              const double* __restrict__ tht, const double* __restrict__ bt, double* __restrict__ F) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)Nt * Ns) return;
  const int s = int(idx / Ns), i = int(idx % Ns);
  int lk[3];
  int sg[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    lk[k] = hop_link[size_t(k) * Ns + i];
    sg[k] = hop_sign[size_t(k) * Ns + i];  // +1: this site is the link's start
  }
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2 - a; b++)
      if (lk[b] > lk[b + 1]) {
        const int tl = lk[b], ts = sg[b];
        lk[b] = lk[b + 1];
        sg[b] = sg[b + 1];
        lk[b + 1] = tl;
        sg[b + 1] = ts;
      }
  double v = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double g = bt[lk[k]] * tht[size_t(s) * Nl + lk[k]];
    if (sg[k] < 0) v += g;
    else v -= g;
  }
  F[size_t(Nt) * Nl + size_t(s) * Ns + perm[i]] = v;
}

__global__ void k_ext_polyakov(int Nt, int Nl, int Ns, const double* __restrict__ A, double* __restrict__ P) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= Ns) return;
  double a = 0.0;
  for (int s = 0; s < Nt; s++) a += A[size_t(Nt) * Nl + size_t(s) * Ns + x];
  double sn, cs;
  sincos(a, &sn, &cs);
  P[2 * x] = cs;
  P[2 * x + 1] = sn;
}

struct ExtBuf {
  double *ths = nullptr, *tht = nullptr, *bs = nullptr, *bt = nullptr;
  ~ExtBuf() {
    for (double* p : {ths, tht, bs, bt})
      if (p) cudaFree(p);
  }
};

static int ext_prepare(qed3_lattice_s* lat, int Nt, double at, double gsq, const double* A, ExtBuf& b,
                       cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  const HostLattice& L = lat->host;
  const DeviceLattice& D = lat->dev;
  const int Nl = D.Nl, Nf = D.Nf, Ns = D.Ns;
  std::vector<double> bs(Nf, 0.0), bt(Nl, 0.0);
  if (std::abs(gsq) > 1.0e-15) {  // U1WilsonExt::set_beta (src/both_3d/action_ext.h:148-158)
    for (int f = 0; f < Nf; f++) bs[f] = at / L.vols[f] / gsq;
    for (int l = 0; l < Nl; l++) bt[l] = 2.0 / at * L.link_volume[l] / std::pow(L.ell[l], 2) / gsq;
  }
  QED3_CUDA_TRY(cudaMalloc(&b.ths, size_t(Nt) * Nf * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&b.tht, size_t(Nt) * Nl * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&b.bs, size_t(Nf) * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&b.bt, size_t(Nl) * sizeof(double)));
  QED3_CUDA_TRY(cudaMemcpyAsync(b.bs, bs.data(), Nf * sizeof(double), cudaMemcpyHostToDevice, st));
  QED3_CUDA_TRY(cudaMemcpyAsync(b.bt, bt.data(), Nl * sizeof(double), cudaMemcpyHostToDevice, st));
  const long long n = (long long)Nt * (Nf + Nl);
  k_ext_plaq<<<nblk(n), 256, 0, st>>>(Nt, Nl, Ns, Nf, D.face_off, D.face_link, D.face_sign, D.link_x, D.link_y,
                                      D.perm, A, b.ths, b.tht);
  QED3_CUDA_TRY(cudaGetLastError());
  QED3_CUDA_TRY(cudaStreamSynchronize(st));  // the host staging vectors go out of scope
  return QED3_OK;
}

int ext_plaquettes(qed3_lattice_s* lat, int Nt, const double* A, double* ths, double* tht, cudaStream_t st) {
  ExtBuf b;
  int rc = ext_prepare(lat, Nt, 1.0, 0.0, A, b, st);
  if (rc) return rc;
  const DeviceLattice& D = lat->dev;
  if (ths) QED3_CUDA_TRY(cudaMemcpyAsync(ths, b.ths, size_t(Nt) * D.Nf * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (tht) QED3_CUDA_TRY(cudaMemcpyAsync(tht, b.tht, size_t(Nt) * D.Nl * sizeof(double), cudaMemcpyDeviceToDevice, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  return QED3_OK;
}

int ext_gauge_action(qed3_lattice_s* lat, int Nt, double at, double gsq, const double* A, double* S, cudaStream_t st) {
  ExtBuf b;
  int rc = ext_prepare(lat, Nt, at, gsq, A, b, st);
  if (rc) return rc;
  const DeviceLattice& D = lat->dev;
  const long long nsp = (long long)Nt * D.Nf;
  return reduce(int(nsp + (long long)Nt * D.Nl), ExtAction{b.ths, b.tht, b.bs, b.bt, nsp, D.Nf, D.Nl},
                lat->gauge.part, S, st);
}

int ext_gauge_force(qed3_lattice_s* lat, int Nt, double at, double gsq, const double* A, double* F, cudaStream_t st) {
  ExtBuf b;
  int rc = ext_prepare(lat, Nt, at, gsq, A, b, st);
  if (rc) return rc;
  const DeviceLattice& D = lat->dev;
  const GaugeDev& G = lat->gauge;
  k_ext_force_s<<<nblk((long long)Nt * D.Nl), 256, 0, st>>>(Nt, D.Nl, D.Nf, G.link_face, G.link_fsign, b.ths, b.tht,
                                                           b.bs, b.bt, F);
  k_ext_force_t<<<nblk((long long)Nt * D.Ns), 256, 0, st>>>(Nt, D.Nl, D.Ns, D.hop_link, D.hop_sign, D.perm, b.tht,
                                                           b.bt, F);
  QED3_CUDA_TRY(cudaGetLastError());
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  return QED3_OK;
}

int ext_polyakov(qed3_lattice_s* lat, int Nt, const double* A, double* P, double* avg, cudaStream_t st) {
  int rc = gauge_prepare(lat);
  if (rc) return rc;
  const DeviceLattice& D = lat->dev;
  double* buf = P;
  if (!buf) QED3_CUDA_TRY(cudaMalloc(&buf, size_t(D.Ns) * 2 * sizeof(double)));
  k_ext_polyakov<<<nblk(D.Ns), 256, 0, st>>>(Nt, D.Nl, D.Ns, A, buf);
  QED3_CUDA_TRY(cudaGetLastError());
  if (avg) {
    std::vector<double> h(size_t(D.Ns) * 2);
    QED3_CUDA_TRY(cudaMemcpyAsync(h.data(), buf, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    QED3_CUDA_TRY(cudaStreamSynchronize(st));
    double re = 0, im = 0;
    for (int x = 0; x < D.Ns; x++) {
      re += h[2 * x];
      im += h[2 * x + 1];
    }
    avg[0] = re / D.Ns;
    avg[1] = im / D.Ns;
  }
  if (!P) cudaFree(buf);
  return QED3_OK;
}

}  // namespace qed3
