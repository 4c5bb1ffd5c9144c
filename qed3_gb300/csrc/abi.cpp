// extern "C" entry points of include/qed3.h.  No exception crosses this
// boundary: every call returns a status and records a message for
// qed3_last_error_string().

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "batched_impl.h"
#include "dirac_impl.h"
#include "gauge_impl.h"
#include "handles.h"
#include "lpc_impl.h"
#include "mshift_impl.h"
#include "ext_impl.h"
#include "overlap_impl.h"
#include "pcg_impl.h"
#include "qed3_internal.h"

namespace qed3 {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

template <class T>
static int upload(T** dst, const std::vector<T>& src) {
  QED3_CUDA_TRY(cudaMalloc(dst, src.size() * sizeof(T) + 16));
  QED3_CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return QED3_OK;
}

int lattice_upload(qed3_lattice_s* lat) {
  const HostLattice& L = lat->host;
  DeviceLattice& D = lat->dev;
  const int Ns = L.n_sites, Nl = L.n_links, Nf = L.n_faces;
  D.Ns = Ns;
  D.Nl = Nl;
  D.Nf = Nf;
  D.face_total = int(L.face_sites.size());
  std::vector<int32_t> nbr(size_t(3) * Ns), nbr_ref(size_t(3) * Ns), hop_link(size_t(3) * Ns);
  std::vector<int8_t> hop_sign(size_t(3) * Ns);
  for (int i = 0; i < Ns; i++) {
    const int x = L.perm[i];
    for (int k = 0; k < 3; k++) {
      const int y = L.nns[3 * x + k];
      nbr[size_t(k) * Ns + i] = L.iperm[y];
      nbr_ref[size_t(k) * Ns + i] = y;
      hop_link[size_t(k) * Ns + i] = L.hop_link[3 * x + k];
      hop_sign[size_t(k) * Ns + i] = L.hop_sign[3 * x + k];
    }
  }
  std::vector<int32_t> link_x(Nl), link_y(Nl);
  std::vector<int8_t> link_kx(Nl), link_ky(Nl);
  for (int l = 0; l < Nl; l++) {
    const int x = L.links[2 * l], y = L.links[2 * l + 1];
    link_x[l] = L.iperm[x];
    link_y[l] = L.iperm[y];
    int kx = 0, ky = 0;
    while (L.nns[3 * x + kx] != y) kx++;
    while (L.nns[3 * y + ky] != x) ky++;
    link_kx[l] = int8_t(kx);
    link_ky[l] = int8_t(ky);
  }
  std::vector<double> fw(Nf);
  for (int f = 0; f < Nf; f++) fw[f] = L.mean_vol / L.vols[f];
  int rc;
  if ((rc = upload(&D.nbr, nbr)) || (rc = upload(&D.nbr_ref, nbr_ref)) || (rc = upload(&D.perm, L.perm)) ||
      (rc = upload(&D.iperm, L.iperm)) || (rc = upload(&D.hop_link, hop_link)) || (rc = upload(&D.hop_sign, hop_sign)) ||
      (rc = upload(&D.face_off, L.face_offsets)) || (rc = upload(&D.face_link, L.face_links)) ||
      (rc = upload(&D.face_sign, L.face_link_sign)) || (rc = upload(&D.face_weight, fw)) ||
      (rc = upload(&D.link_x, link_x)) || (rc = upload(&D.link_y, link_y)) || (rc = upload(&D.link_kx, link_kx)) ||
      (rc = upload(&D.link_ky, link_ky)))
    return rc;
  return QED3_OK;
}

int lattice_free(qed3_lattice_s* lat) {
  DeviceLattice& D = lat->dev;
  void* ptrs[] = {D.nbr, D.nbr_ref, D.perm, D.iperm, D.hop_link, D.hop_sign, D.face_off, D.face_link,
                  D.face_sign, D.face_weight, D.link_x, D.link_y, D.link_kx, D.link_ky};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  D = DeviceLattice{};
  return QED3_OK;
}

}  // namespace qed3

using namespace qed3;

#define QED3_GUARD_BEGIN try {
#define QED3_GUARD_END                                                   \
  }                                                                      \
  catch (const std::bad_alloc&) {                                        \
    return fail(QED3_ERR_NOMEM, "host allocation failed");               \
  }                                                                      \
  catch (const std::exception& e) {                                      \
    return fail(QED3_ERR_STATE, std::string("internal error: ") + e.what()); \
  }                                                                      \
  catch (...) {                                                          \
    return fail(QED3_ERR_STATE, "internal error");                       \
  }

extern "C" {

const char* qed3_last_error_string(void) { return g_last_error.c_str(); }
int qed3_version(void) { return 100; }

int qed3_selftest_wait_timeout(long long spin_limit, int* timed_out_resident, int* timed_out_streaming) {
  QED3_GUARD_BEGIN
  return selftest_wait_timeout(spin_limit, timed_out_resident, timed_out_streaming);
  QED3_GUARD_END
}

int qed3_lattice_create(int n_refine, qed3_lattice** out) {
  QED3_GUARD_BEGIN
  if (!out) return fail(QED3_ERR_ARG, "out is NULL");
  *out = nullptr;
  auto* lat = new qed3_lattice_s;
  int rc = build_lattice(n_refine, true, lat->host);
  if (rc) {
    delete lat;
    return rc;
  }
  // device tables are uploaded on first device use (qed3_dirac_create, gauge
  // kernels), so host-only queries need no GPU
  *out = lat;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_lattice_from_mesh(int n_vertices, const double* vertices, int n_triangles, const int* triangles,
                           const int* links, qed3_lattice** out) {
  QED3_GUARD_BEGIN
  if (!out || !vertices || !triangles) return fail(QED3_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* lat = new qed3_lattice_s;
  int rc = build_lattice_from_mesh(n_vertices, vertices, n_triangles, triangles, links, true, lat->host);
  if (rc) {
    delete lat;
    return rc;
  }
  *out = lat;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_lattice_mesh(const qed3_lattice* lat, double* vertices, int* triangles) {
  if (!lat) return fail(QED3_ERR_ARG, "lattice is NULL");
  const HostLattice& L = lat->host;
  if (vertices) std::memcpy(vertices, L.simp_sites.data(), L.simp_sites.size() * sizeof(double));
  if (triangles) std::memcpy(triangles, L.simp_faces.data(), L.simp_faces.size() * sizeof(int32_t));
  return QED3_OK;
}

int qed3_lattice_set_spin_structure(qed3_lattice* lat, const double* omega, const double* alpha) {
  if (!lat) return fail(QED3_ERR_ARG, "lattice is NULL");
  HostLattice& L = lat->host;
  for (int pass = 0; pass < 2; pass++) {  // check everything before changing anything
    const double* src = pass == 0 ? omega : alpha;
    const size_t n = pass == 0 ? L.omega.size() : L.alpha.size();
    if (!src) continue;
    for (size_t i = 0; i < n; i++)
      if (!std::isfinite(src[i])) return fail(QED3_ERR_ARG, "spin structure: non-finite entry");
  }
  if (omega) std::memcpy(L.omega.data(), omega, L.omega.size() * sizeof(double));
  if (alpha) std::memcpy(L.alpha.data(), alpha, L.alpha.size() * sizeof(double));
  return QED3_OK;
}

int qed3_lattice_destroy(qed3_lattice* lat) {
  if (!lat) return QED3_OK;
  gauge_free(lat);
  lattice_free(lat);
  delete lat;
  return QED3_OK;
}

int qed3_lattice_sizes(const qed3_lattice* lat, int* n_sites, int* n_links, int* n_faces, int* face_total) {
  if (!lat) return fail(QED3_ERR_ARG, "lattice is NULL");
  if (n_sites) *n_sites = lat->host.n_sites;
  if (n_links) *n_links = lat->host.n_links;
  if (n_faces) *n_faces = lat->host.n_faces;
  if (face_total) *face_total = int(lat->host.face_sites.size());
  return QED3_OK;
}

int qed3_lattice_tables(const qed3_lattice* lat, double* sites, int* nns, int* links, int* simp_links,
                        int* face_offsets, int* face_sites, double* ell, double* link_volume, double* vols,
                        double* omega, double* alpha, double* means) {
  if (!lat) return fail(QED3_ERR_ARG, "lattice is NULL");
  const HostLattice& L = lat->host;
  auto cp = [](auto* dst, const auto& v) {
    if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(sites, L.sites);
  cp(nns, L.nns);
  cp(links, L.links);
  cp(simp_links, L.simp_links);
  cp(face_offsets, L.face_offsets);
  cp(face_sites, L.face_sites);
  cp(ell, L.ell);
  cp(link_volume, L.link_volume);
  cp(vols, L.vols);
  cp(omega, L.omega);
  cp(alpha, L.alpha);
  if (means) {
    means[0] = L.mean_ell;
    means[1] = L.mean_link_volume;
    means[2] = L.mean_vol;
  }
  return QED3_OK;
}

int qed3_lattice_permutation(const qed3_lattice* lat, int* perm) {
  if (!lat || !perm) return fail(QED3_ERR_ARG, "NULL argument");
  std::memcpy(perm, lat->host.perm.data(), lat->host.perm.size() * sizeof(int32_t));
  return QED3_OK;
}

int qed3_dirac_create_1f(qed3_lattice* lat, double r, double m, double M5, qed3_dirac** out) {
  QED3_GUARD_BEGIN
  if (!lat || !out) return fail(QED3_ERR_ARG, "NULL argument");
  int rc = qed3_dirac_create(lat, r, M5, out);
  if (rc) return rc;
  rc = dirac_use_1f(*out, m);
  if (rc) {
    qed3_dirac_destroy(*out);
    *out = nullptr;
  }
  return rc;
  QED3_GUARD_END
}

int qed3_dirac_create(qed3_lattice* lat, double r, double M5, qed3_dirac** out) {
  QED3_GUARD_BEGIN
  if (!lat || !out) return fail(QED3_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (!lat->dev.nbr) {
    cudaGetDevice(&lat->device);
    int rc0 = lattice_upload(lat);
    if (rc0) {
      lattice_free(lat);
      return rc0;
    }
  }
  auto* d = new qed3_dirac_s;
  d->lat = lat;
  d->r = r;
  d->M5 = M5;
  int rc = dirac_init_device(d);
  if (rc) {
    dirac_free_device(d);
    delete d;
    return rc;
  }
  *out = d;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_dirac_ext_create(qed3_lattice* lat, double r, double M5, int Nt, double at, qed3_dirac_ext** out) {
  QED3_GUARD_BEGIN
  if (!lat || !out) return fail(QED3_ERR_ARG, "NULL argument");
  if (Nt < 1 || Nt > 4096 || !(at > 0)) return fail(QED3_ERR_ARG, "need 1 <= Nt <= 4096 and at > 0");
  *out = nullptr;
  qed3_dirac* d2 = nullptr;
  int rc = qed3_dirac_create(lat, r, M5, &d2);
  if (rc) return rc;
  auto* e = new qed3_dirac_ext_s;
  e->d2 = d2;
  e->Nt = Nt;
  e->at = at;
  e->r = r;
  if ((rc = ext_init(e))) {
    ext_free(e);
    qed3_dirac_destroy(d2);
    delete e;
    return rc;
  }
  *out = e;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_dirac_ext_destroy(qed3_dirac_ext* e) {
  if (!e) return QED3_OK;
  ext_free(e);
  qed3_dirac_destroy(e->d2);
  delete e;
  return QED3_OK;
}

int qed3_dirac_ext_set_links(qed3_dirac_ext* e, const double* A, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !A) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_set_links(e, A, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_ext_apply(qed3_dirac_ext* e, int op, double* out, const double* in, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !out || !in) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_apply(e, op, out, in, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_ext_fermion_force(qed3_dirac_ext* e, const double* eta, double* F, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !eta || !F) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_fermion_force(e, eta, F, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_ext_force(qed3_overlap_ext* ov, const double* eta, double* F, double tol_inner, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !eta || !F) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_overlap_force(ov, eta, F, tol_inner > 0 ? tol_inner : 1e-12, nullptr, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_hmc_ext_overlap(qed3_overlap_ext* ov, qed3_rng* rng, double* A, double at, double gsq, double tmax,
                         int nsteps, int nsteps_inner, int npf, int integrator, double tol, double tol_inner,
                         double lambda_min, double lambda_max, int no_reject, int* accepted, double* dH,
                         int* cg_iters, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !rng || !A || !accepted || !dH) return fail(QED3_ERR_ARG, "NULL argument");
  qed3_dirac_ext_s* e = ext_overlap_operator(ov);
  if (nsteps < 1 || nsteps_inner < 1 || !(tmax > 0) || npf < 1 || npf > 64 || !(at > 0))
    return fail(QED3_ERR_ARG, "need nsteps, nsteps_inner, npf >= 1, tmax > 0, at > 0");
  if (integrator != QED3_INTEGRATOR_LEAPFROG_ML && integrator != QED3_INTEGRATOR_LEAPFROG)
    return fail(QED3_ERR_ARG, "unknown integrator");
  const size_t nl = size_t(e->d2->lat->host.n_links) * e->Nt, ns = size_t(e->d2->Ns) * e->Nt;
  size_t rl = 0, rs = 0;
  rng_counts(rng, &rl, &rs);
  if (rl != nl || rs != ns)
    return fail(QED3_ERR_ARG, "rng must hold Nt n_links link engines and Nt n_sites site engines");
  if ((lambda_min > 0) != (lambda_max > 0)) return fail(QED3_ERR_ARG, "fix both bounds or neither");
  return hmc_ext(e, rng, A, at, gsq, tmax, nsteps, nsteps_inner, npf, integrator, tol > 0 ? tol : 1e-10,
                 QED3_PREC_F64, no_reject, accepted, dH, cg_iters, (cudaStream_t)stream, ov,
                 tol_inner > 0 ? tol_inner : 1e-12, lambda_min, lambda_max);
  QED3_GUARD_END
}

int qed3_hmc_ext(qed3_dirac_ext* e, qed3_rng* rng, double* A, double at, double gsq, double tmax, int nsteps,
                 int nsteps_inner, int npf, int integrator, double tol, int precision, int no_reject, int* accepted,
                 double* dH, int* cg_iters, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !rng || !A || !accepted || !dH) return fail(QED3_ERR_ARG, "NULL argument");
  if (nsteps < 1 || nsteps_inner < 1 || !(tmax > 0) || npf < 1 || npf > 64 || !(at > 0))
    return fail(QED3_ERR_ARG, "need nsteps, nsteps_inner, npf >= 1, tmax > 0, at > 0");
  if (integrator != QED3_INTEGRATOR_LEAPFROG_ML && integrator != QED3_INTEGRATOR_LEAPFROG)
    return fail(QED3_ERR_ARG, "unknown integrator");
  const size_t nl = size_t(e->d2->lat->host.n_links) * e->Nt, ns = size_t(e->d2->Ns) * e->Nt;
  size_t rl = 0, rs = 0;
  rng_counts(rng, &rl, &rs);
  if (rl != nl || rs != ns)
    return fail(QED3_ERR_ARG, "rng must hold Nt n_links link engines and Nt n_sites site engines");
  if (precision != QED3_PREC_F64 && precision != QED3_PREC_F32) return fail(QED3_ERR_ARG, "precision F64 or F32");
  return hmc_ext(e, rng, A, at, gsq, tmax, nsteps, nsteps_inner, npf, integrator, tol > 0 ? tol : 1e-10, precision,
                 no_reject, accepted, dH, cg_iters, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_ext_propagator(qed3_dirac_ext* e, int s, int ix, int a, int dagger, double* sink, const qed3_solve_params* params,
                              qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !sink) return fail(QED3_ERR_ARG, "NULL argument");
  qed3_solve_params p{params ? params->tol : 1e-10, params ? params->maxiter : 0,
                      params && params->precision == QED3_PREC_F32 ? QED3_PREC_F32 : QED3_PREC_F64,
                      params && params->delta > 0 ? params->delta : 0.1, 0.0, 0};
  return ext_propagator(e, s, ix, a, dagger, sink, &p, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_ext_create(qed3_dirac_ext* e, int order, qed3_overlap_ext** out) {
  QED3_GUARD_BEGIN
  if (!e || !out) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_overlap_create(e, order, out);
  QED3_GUARD_END
}

int qed3_overlap_ext_destroy(qed3_overlap_ext* ov) {
  QED3_GUARD_BEGIN
  ext_overlap_destroy(ov);
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_overlap_ext_update(qed3_overlap_ext* ov, double lambda_min, double lambda_max, double tol, double margin,
                            void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !(margin >= 0 && margin < 0.5)) return fail(QED3_ERR_ARG, "bad argument");
  return ext_overlap_update(ov, lambda_min, lambda_max, tol, margin, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_ext_info(const qed3_overlap_ext* ov, double* lambda_min, double* lambda_max, double* k,
                          double* delta) {
  QED3_GUARD_BEGIN
  if (!ov || !lambda_min || !lambda_max || !k || !delta) return fail(QED3_ERR_ARG, "NULL argument");
  ext_overlap_info(ov, lambda_min, lambda_max, k, delta);
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_overlap_ext_apply(qed3_overlap_ext* ov, int op, double* out, const double* in, double tol_inner,
                           int* pole_iters, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !out || !in || out == in) return fail(QED3_ERR_ARG, "NULL or aliased argument");
  return ext_overlap_apply(ov, op, out, in, tol_inner > 0 ? tol_inner : 1e-12, pole_iters, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_ext_solve(qed3_overlap_ext* ov, double* x, const double* b, double tol, double tol_inner,
                           int maxiter, int prop, qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !x || !b || x == b) return fail(QED3_ERR_ARG, "NULL or aliased argument");
  return ext_overlap_solve(ov, x, b, tol > 0 ? tol : 1e-10, tol_inner > 0 ? tol_inner : 1e-12,
                           maxiter > 0 ? maxiter : 100000, prop, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_ext_cg_solve(qed3_dirac_ext* e, double* x, const double* b, const qed3_solve_params* params,
                            qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!e || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  return ext_cg(e, x, b, params, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_ext_plaquettes(qed3_lattice* lat, int Nt, const double* A, double* theta_s, double* theta_t, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || Nt < 1) return fail(QED3_ERR_ARG, "bad argument");
  return ext_plaquettes(lat, Nt, A, theta_s, theta_t, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_ext_gauge_action(qed3_lattice* lat, int Nt, double at, double gsq, const double* A, double* S, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !S || Nt < 1 || !(at > 0)) return fail(QED3_ERR_ARG, "bad argument");
  return ext_gauge_action(lat, Nt, at, gsq, A, S, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_ext_gauge_force(qed3_lattice* lat, int Nt, double at, double gsq, const double* A, double* F, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !F || Nt < 1 || !(at > 0)) return fail(QED3_ERR_ARG, "bad argument");
  return ext_gauge_force(lat, Nt, at, gsq, A, F, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_ext_polyakov(qed3_lattice* lat, int Nt, const double* A, double* P, double* avg, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || Nt < 1) return fail(QED3_ERR_ARG, "bad argument");
  return ext_polyakov(lat, Nt, A, P, avg, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_destroy(qed3_dirac* d) {
  if (!d) return QED3_OK;
  solver_free(d);
  dirac_free_device(d);
  delete d;
  return QED3_OK;
}

int qed3_dirac_set_links(qed3_dirac* d, const double* A, int A_on_device, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !A) return fail(QED3_ERR_ARG, "NULL argument");
  return dirac_set_links(d, A, A_on_device, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_set_coefficients(qed3_dirac* d, const double* hop, const double* diag) {
  QED3_GUARD_BEGIN
  if (!d || !hop || !diag) return fail(QED3_ERR_ARG, "NULL argument");
  return dirac_set_coefficients(d, hop, diag);
  QED3_GUARD_END
}

int qed3_dirac_apply(qed3_dirac* d, int op, double* out, const double* in, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !out || !in) return fail(QED3_ERR_ARG, "NULL argument");
  if (op < QED3_OP_D || op > QED3_OP_DDDAG) return fail(QED3_ERR_ARG, "unknown operator");
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  return dirac_apply_ref(d, op, out, in, (cudaStream_t)stream);
  QED3_GUARD_END
}

size_t qed3_field_bytes(const qed3_dirac* d, int prec, int nrhs) {
  if (!d || nrhs < 1) return 0;
  const size_t per = prec == QED3_PREC_F64 ? 32 : prec == QED3_PREC_F32 ? 16 : 8;
  return per * size_t(d->Ns) * size_t(nrhs);
}

int qed3_field_import(qed3_dirac* d, int prec, void* field, const double* in_ref, int nrhs, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !field || !in_ref || nrhs < 1) return fail(QED3_ERR_ARG, "bad argument");
  if (prec < 0 || prec > 2) return fail(QED3_ERR_ARG, "unknown precision");
  return field_import(d, prec, field, in_ref, nrhs, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_field_export(qed3_dirac* d, int prec, double* out_ref, const void* field, int nrhs, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !field || !out_ref || nrhs < 1) return fail(QED3_ERR_ARG, "bad argument");
  if (prec < 0 || prec > 2) return fail(QED3_ERR_ARG, "unknown precision");
  return field_export(d, prec, out_ref, field, nrhs, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_apply_field(qed3_dirac* d, int op, int prec, void* out, const void* in, int nrhs, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !out || !in || nrhs < 1) return fail(QED3_ERR_ARG, "bad argument");
  if (prec < 0 || prec > 2) return fail(QED3_ERR_ARG, "unknown precision");
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  if (out == in) return fail(QED3_ERR_ARG, "the stencil gathers: out must not alias in");
  return dirac_apply_field(d, op, prec, out, in, nrhs, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_cg_solve(qed3_dirac* d, double* x, const double* b, const qed3_solve_params* params,
                  qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  return cg_solve(d, x, b, params, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_cg_solve_noalloc(qed3_dirac* d, double* x, const double* b, const qed3_solve_params* params,
                          qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  return cg_solve_noalloc(d, x, b, params, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_bicgstab_solve(qed3_dirac* d, int op, double* x, const double* b, const qed3_solve_params* params,
                        double eps, qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  return bicgstab_solve(d, op, x, b, params, eps, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_dirac_spectral_bounds(qed3_dirac* d, double tol, int maxsteps, double* lambda_min, double* lambda_max,
                               int* steps, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !lambda_min || !lambda_max) return fail(QED3_ERR_ARG, "NULL argument");
  return spectral_bounds(d, tol, maxsteps, lambda_min, lambda_max, steps, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_solver_last_report(qed3_dirac* d, qed3_solve_report* report) {
  if (!d || !report) return fail(QED3_ERR_ARG, "NULL argument");
  *report = d->last;
  return QED3_OK;
}

int qed3_plaquette(qed3_lattice* lat, const double* A, double* theta, double* avg, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A) return fail(QED3_ERR_ARG, "NULL argument");
  return gauge_plaquette_avg(lat, A, theta, avg, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_gauge_action(qed3_lattice* lat, const double* A, double beta, int compact, double* S, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !S) return fail(QED3_ERR_ARG, "NULL argument");
  return gauge_action(lat, A, beta, compact, S, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_gauge_force(qed3_lattice* lat, const double* A, double beta, int compact, int exact, double* F, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !F) return fail(QED3_ERR_ARG, "NULL argument");
  return gauge_force(lat, A, beta, compact, exact, F, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_fermion_force(qed3_dirac* d, const double* eta, double* F, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !eta || !F) return fail(QED3_ERR_ARG, "NULL argument");
  return fermion_force(d, eta, F, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_rng_create(int n_links, int n_sites, int seed, qed3_rng** out) {
  QED3_GUARD_BEGIN
  if (!out || n_links < 0 || n_sites < 0) return fail(QED3_ERR_ARG, "bad argument");
  *out = rng_create(n_links, n_sites, seed);
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_rng_destroy(qed3_rng* r) {
  rng_destroy(r);
  return QED3_OK;
}

int qed3_rng_uniform(qed3_rng* r, double* out) {
  if (!r || !out) return fail(QED3_ERR_ARG, "NULL argument");
  *out = rng_uniform(r);
  return QED3_OK;
}

int qed3_rng_save(const qed3_rng* r, const char* path) {
  QED3_GUARD_BEGIN
  if (!r || !path) return fail(QED3_ERR_ARG, "NULL argument");
  return rng_save(r, path);
  QED3_GUARD_END
}

int qed3_rng_load(qed3_rng* r, const char* path) {
  QED3_GUARD_BEGIN
  if (!r || !path) return fail(QED3_ERR_ARG, "NULL argument");
  return rng_load(r, path);
  QED3_GUARD_END
}

// GaugeExt::ckpoint / read (src/both_3d/gauge_ext.h:225-275) at Nt = 1: raw
// native-endian doubles, the spatial links [n_links] then the temporal links
// [n_sites] (zero here: the dual-lattice path has no temporal direction).
int qed3_links_save(const qed3_lattice* lat, const double* A, const char* path) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !path) return fail(QED3_ERR_ARG, "NULL argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(QED3_ERR_ARG, std::string("cannot write ") + path);
  const size_t nl = size_t(lat->host.n_links), ns = size_t(lat->host.n_sites);
  std::vector<double> zeros(ns, 0.0);
  const bool ok = std::fwrite(A, sizeof(double), nl, f) == nl && std::fwrite(zeros.data(), sizeof(double), ns, f) == ns;
  std::fclose(f);
  return ok ? QED3_OK : fail(QED3_ERR_ARG, std::string("write failed: ") + path);
  QED3_GUARD_END
}

int qed3_links_load(const qed3_lattice* lat, double* A, double* temporal_max_abs, const char* path) {
  QED3_GUARD_BEGIN
  if (!lat || !A || !path) return fail(QED3_ERR_ARG, "NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(QED3_ERR_ARG, std::string("cannot read ") + path);
  const size_t nl = size_t(lat->host.n_links), ns = size_t(lat->host.n_sites);
  std::vector<double> buf(nl + ns + 1);
  const size_t got = std::fread(buf.data(), sizeof(double), nl + ns + 1, f);
  std::fclose(f);
  if (got != nl + ns) return fail(QED3_ERR_ARG, "not a gauge checkpoint of this lattice (Nt = 1): " + std::string(path));
  std::memcpy(A, buf.data(), nl * sizeof(double));
  double mx = 0.0;
  for (size_t i = 0; i < ns; i++) mx = std::max(mx, std::abs(buf[nl + i]));
  if (temporal_max_abs) *temporal_max_abs = mx;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_rng_gaussian_links(qed3_rng* r, double width, double* links) {
  if (!r || !links) return fail(QED3_ERR_ARG, "NULL argument");
  rng_gaussian_links(r, width, links);
  return QED3_OK;
}

int qed3_rng_gaussian_spinor(qed3_rng* r, double* spinor) {
  if (!r || !spinor) return fail(QED3_ERR_ARG, "NULL argument");
  rng_gaussian_spinor(r, spinor);
  return QED3_OK;
}

int qed3_rng_z2_spinor(qed3_rng* r, double* spinor) {
  if (!r || !spinor) return fail(QED3_ERR_ARG, "NULL argument");
  rng_z2_spinor(r, spinor);
  return QED3_OK;
}

int qed3_point_source(int n_sites, int x, int s, double* spinor) {
  if (!spinor || n_sites < 1) return fail(QED3_ERR_ARG, "NULL argument or empty lattice");
  if (x < 0 || x >= n_sites || s < 0 || s > 1) return fail(QED3_ERR_ARG, "site or spin out of range");
  std::memset(spinor, 0, size_t(4) * n_sites * sizeof(double));
  spinor[4 * size_t(x) + 2 * s] = 1.0;
  return QED3_OK;
}

int qed3_hmc_fermion(qed3_lattice* lat, qed3_dirac* d, qed3_rng* rng, double* A, double beta, int compact, int exact,
                     double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double tol, int precision,
                     int no_reject, int* accepted, double* dH, int* cg_iters, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !d || !rng || !A || !accepted || !dH) return fail(QED3_ERR_ARG, "NULL argument");
  if (d->lat != lat) return fail(QED3_ERR_ARG, "operator belongs to another lattice");
  if (nsteps < 1 || nsteps_inner < 1 || !(tmax > 0)) return fail(QED3_ERR_ARG, "need nsteps, nsteps_inner >= 1, tmax > 0");
  if (precision < 0 || precision > 2) return fail(QED3_ERR_ARG, "unknown precision");
  if (npf < 1 || npf > 64) return fail(QED3_ERR_ARG, "need 1 <= npf <= 64 pseudofermions");
  if (integrator != QED3_INTEGRATOR_LEAPFROG_ML && integrator != QED3_INTEGRATOR_LEAPFROG)
    return fail(QED3_ERR_ARG, "unknown integrator");
  return hmc_fermion(lat, d, rng, A, beta, compact, exact, tmax, nsteps, nsteps_inner, npf, integrator,
                     tol > 0 ? tol : 1e-10, precision, no_reject, accepted, dH, cg_iters, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_hmc_overlap(qed3_lattice* lat, qed3_overlap* ov, qed3_rng* rng, double* A, double beta, int compact,
                     int exact, double tmax, int nsteps, int nsteps_inner, int npf, int integrator, double lmin,
                     double lmax, double tol, double tol_inner, int no_reject, int* accepted, double* dH,
                     int* cg_iters, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !ov || !rng || !A || !accepted || !dH) return fail(QED3_ERR_ARG, "NULL argument");
  if (overlap_dirac(ov)->lat != lat) return fail(QED3_ERR_ARG, "overlap operator belongs to another lattice");
  if (nsteps < 1 || nsteps_inner < 1 || !(tmax > 0)) return fail(QED3_ERR_ARG, "need nsteps, nsteps_inner >= 1, tmax > 0");
  if (npf < 1 || npf > 64) return fail(QED3_ERR_ARG, "need 1 <= npf <= 64 pseudofermions");
  const bool fixed = lmin > 0 || lmax > 0;
  if (fixed && !(lmin > 0 && lmin < lmax)) return fail(QED3_ERR_ARG, "fixed bounds need 0 < lmin < lmax");
  if (integrator != QED3_INTEGRATOR_LEAPFROG_ML && integrator != QED3_INTEGRATOR_LEAPFROG)
    return fail(QED3_ERR_ARG, "unknown integrator");
  return hmc_overlap(lat, ov, rng, A, beta, compact, exact, tmax, nsteps, nsteps_inner, npf, integrator,
                     fixed ? lmin : 0.0, fixed ? lmax : 0.0, tol > 0 ? tol : 1e-10, tol_inner > 0 ? tol_inner : 1e-12,
                     no_reject, accepted, dH, cg_iters, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_hmc_pure_gauge(qed3_lattice* lat, qed3_rng* rng, double* A, double beta, int compact, int exact,
                        double tmax, int nsteps, int no_reject, int* accepted, double* dH, void* stream) {
  QED3_GUARD_BEGIN
  if (!lat || !rng || !A || !accepted || !dH || nsteps < 1) return fail(QED3_ERR_ARG, "bad argument");
  return hmc_pure_gauge(lat, rng, A, beta, compact, exact, tmax, nsteps, no_reject, accepted, dH,
                        (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_batch_create(int nsys, qed3_dirac* const* ops, const int* nrhs, int precision, int rhs_tile, int threads,
                      qed3_batch** out) {
  QED3_GUARD_BEGIN
  if (!out || !ops || !nrhs || nsys < 1) return fail(QED3_ERR_ARG, "bad argument");
  if (precision < 0 || precision > 2) return fail(QED3_ERR_ARG, "unknown precision");
  for (int u = 0; u < nsys; u++)
    if (!ops[u] || nrhs[u] < 1) return fail(QED3_ERR_ARG, "each system needs an operator and >= 1 rhs");
  *out = nullptr;
  return batch_create(nsys, ops, nrhs, precision, rhs_tile, threads, out);
  QED3_GUARD_END
}

int qed3_batch_create2(int nsys, qed3_dirac* const* ops, const int* nrhs, int precision, int rhs_tile, int threads,
                       int schedule, qed3_batch** out) {
  QED3_GUARD_BEGIN
  if (!out || !ops || !nrhs || nsys < 1) return fail(QED3_ERR_ARG, "bad argument");
  if (precision < 0 || precision > 2) return fail(QED3_ERR_ARG, "unknown precision");
  for (int u = 0; u < nsys; u++)
    if (!ops[u] || nrhs[u] < 1) return fail(QED3_ERR_ARG, "each system needs an operator and >= 1 rhs");
  *out = nullptr;
  return batch_create(nsys, ops, nrhs, precision, rhs_tile, threads, out, schedule);
  QED3_GUARD_END
}

int qed3_batch_schedule(const qed3_batch* bt, int* schedule) {
  if (!bt || !schedule) return fail(QED3_ERR_ARG, "NULL argument");
  *schedule = bt->sched;
  return QED3_OK;
}

int qed3_batch_destroy(qed3_batch* bt) {
  batch_destroy(bt);
  return QED3_OK;
}

int qed3_batch_config(const qed3_batch* bt, int* rhs_tile, int* threads, int* blocks) {
  if (!bt) return fail(QED3_ERR_ARG, "NULL batch");
  if (rhs_tile) *rhs_tile = bt->R;
  if (threads) *threads = bt->threads;
  if (blocks) *blocks = bt->grid;
  return QED3_OK;
}

int qed3_batch_solve(qed3_batch* bt, double* const* x, const double* const* b, const double* const* shifts,
                     const qed3_solve_params* params, qed3_solve_report* reports, float* ms, void* stream) {
  QED3_GUARD_BEGIN
  if (!bt || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  for (size_t u = 0; u < bt->user_ops.size(); u++)
    if (!x[u] || !b[u]) return fail(QED3_ERR_ARG, "NULL vector");
  return batch_solve(bt, x, b, shifts, params, reports, ms, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_batch_set_shifts(qed3_batch* bt, const double* const* shifts, double shift, void* stream) {
  QED3_GUARD_BEGIN
  if (!bt) return fail(QED3_ERR_ARG, "NULL argument");
  return batch_set_shifts(bt, shifts, shift, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_batch_launch(qed3_batch* bt, double* const* x, const double* const* b, const qed3_solve_params* params,
                      void* stream) {
  QED3_GUARD_BEGIN
  if (!bt || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  for (size_t u = 0; u < bt->user_ops.size(); u++)
    if (!x[u] || !b[u]) return fail(QED3_ERR_ARG, "NULL vector");
  return batch_launch_all(bt, x, b, params, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_batch_reports(qed3_batch* bt, qed3_solve_report* reports, void* stream) {
  QED3_GUARD_BEGIN
  if (!bt) return fail(QED3_ERR_ARG, "NULL argument");
  return batch_reports(bt, reports, 0.f, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_create(qed3_dirac* dw, int zolo_order, int precision, qed3_overlap** out) {
  QED3_GUARD_BEGIN
  if (!dw || !out) return fail(QED3_ERR_ARG, "NULL argument");
  if (precision < 0 || precision > 2) return fail(QED3_ERR_ARG, "unknown precision");
  *out = nullptr;
  return overlap_create(dw, zolo_order, precision, out);
  QED3_GUARD_END
}

int qed3_overlap_destroy(qed3_overlap* ov) {
  overlap_destroy(ov);
  return QED3_OK;
}

int qed3_overlap_update(qed3_overlap* ov, double lambda_min, double lambda_max, double tol_outer, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov) return fail(QED3_ERR_ARG, "NULL overlap");
  return overlap_update(ov, lambda_min, lambda_max, tol_outer > 0 ? tol_outer : 1e-8, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_info(const qed3_overlap* ov, double* lambda_min, double* lambda_max, double* k, double* delta,
                      int* npoles, int* npoles_fp64) {
  if (!ov) return fail(QED3_ERR_ARG, "NULL overlap");
  return overlap_info(ov, lambda_min, lambda_max, k, delta, npoles, npoles_fp64);
}

int qed3_overlap_apply(qed3_overlap* ov, int op, double* out, const double* in, double tol_inner,
                       qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !out || !in) return fail(QED3_ERR_ARG, "NULL argument");
  if (op < QED3_OP_D || op > QED3_OP_DDDAG) return fail(QED3_ERR_ARG, "unknown operator");
  if (out == in) return fail(QED3_ERR_ARG, "out must not alias in");
  return overlap_apply(ov, op, out, in, tol_inner > 0 ? tol_inner : 1e-10, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_force(qed3_overlap* ov, const double* eta, double* F, double tol_inner, qed3_solve_report* report,
                       void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !eta || !F) return fail(QED3_ERR_ARG, "NULL argument");
  return overlap_force(ov, eta, F, tol_inner > 0 ? tol_inner : 1e-10, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_solve(qed3_overlap* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                       qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  if (x == b) return fail(QED3_ERR_ARG, "x must not alias b");
  return overlap_solve(ov, x, b, tol > 0 ? tol : 1e-10, tol_inner > 0 ? tol_inner : 1e-12,
                       maxiter > 0 ? maxiter : 10000, 0, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_solve2(qed3_overlap* ov, double* x, const double* b, double tol, double tol_inner, int maxiter,
                        int flags, qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  if (x == b) return fail(QED3_ERR_ARG, "x must not alias b");
  if (flags & ~QED3_OVSOLVE_CHIRAL) return fail(QED3_ERR_ARG, "unknown flags");
  return overlap_solve(ov, x, b, tol > 0 ? tol : 1e-10, tol_inner > 0 ? tol_inner : 1e-12,
                       maxiter > 0 ? maxiter : 10000, flags, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_project_low_modes(qed3_overlap* ov, int nev, double tol, int maxsteps, double margin, void* stream) {
  QED3_GUARD_BEGIN
  if (!ov) return fail(QED3_ERR_ARG, "NULL argument");
  return overlap_project_low_modes(ov, nev, tol > 0 ? tol : 1e-13, maxsteps > 0 ? maxsteps : 6000,
                                   margin >= 0 ? margin : 1e-3, (cudaStream_t)stream);
  QED3_GUARD_END
}

int qed3_overlap_set_mass(qed3_overlap* ov, double mass) {
  QED3_GUARD_BEGIN
  if (!ov) return fail(QED3_ERR_ARG, "NULL argument");
  return overlap_set_mass(ov, mass);
  QED3_GUARD_END
}

int qed3_overlap_set_pole_solver(qed3_overlap* ov, int mode) {
  QED3_GUARD_BEGIN
  if (!ov) return fail(QED3_ERR_ARG, "NULL argument");
  return overlap_set_pole_solver(ov, mode);
  QED3_GUARD_END
}

int qed3_overlap_low_modes_info(const qed3_overlap* ov, int* nev, double* max_residual, int* lanczos_steps,
                                double* mu) {
  QED3_GUARD_BEGIN
  if (!ov) return fail(QED3_ERR_ARG, "NULL argument");
  return overlap_low_modes_info(ov, nev, max_residual, lanczos_steps, mu);
  QED3_GUARD_END
}

int qed3_multishift_solve(qed3_dirac* d, int nshifts, const double* shifts, double* x, const double* b, double tol,
                          int maxiter, qed3_solve_report* reports, float* ms, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !shifts || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  if (nshifts < 1 || nshifts > kMsMaxShifts) return fail(QED3_ERR_ARG, "nshifts must be in [1, 64]");
  const size_t bytes = size_t(nshifts) * d->Ns * 4 * sizeof(double);
  void *X = nullptr, *P = nullptr;
  if (cudaMalloc(&X, bytes) != cudaSuccess) return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  if (cudaMalloc(&P, bytes) != cudaSuccess) {
    cudaFree(X);
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  const int rc = mshift_solve(d, nshifts, shifts, b, x, reinterpret_cast<S64*>(X), reinterpret_cast<S64*>(P),
                              tol > 0 ? tol : 1e-10, maxiter > 0 ? maxiter : 200000, reports, ms,
                              (cudaStream_t)stream);
  cudaFree(X);
  cudaFree(P);
  return rc;
  QED3_GUARD_END
}

int qed3_zolotarev(double k, int n, double* c, double* cp, double* A, double* scal, int* size) {
  QED3_GUARD_BEGIN
  ZoloCoeffs z;
  const int rc = zolotarev_coeffs(k, n, z);
  if (rc) return rc;
  for (int m = 0; m < z.size; m++) {
    if (c) c[m] = z.c[m];
    if (cp) cp[m] = z.cp[m];
    if (A) A[m] = z.A[m];
  }
  if (scal) {
    scal[0] = z.M;
    scal[1] = z.lambda_inv;
    scal[2] = z.E;
    scal[3] = z.C;
  }
  if (size) *size = z.size;
  return QED3_OK;
  QED3_GUARD_END
}

int qed3_lpc_create(qed3_dirac* d, int channels, int layers, unsigned seed, qed3_lpc** out) {
  QED3_GUARD_BEGIN
  if (!d || !out) return fail(QED3_ERR_ARG, "NULL argument");
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  *out = nullptr;
  int dev = 0, smc = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  QED3_CUDA_TRY(cudaDeviceGetAttribute(&smc, cudaDevAttrMultiProcessorCount, dev));
  return lpc_create(d, channels, layers, pcg_block_sites(d->Ns, smc), seed, out);
  QED3_GUARD_END
}

int qed3_lpc_destroy(qed3_lpc* pc) {
  lpc_destroy(pc);
  return QED3_OK;
}

int qed3_lpc_info(const qed3_lpc* pc, int* nparams, int* block_sites, int* npairs) {
  if (!pc) return fail(QED3_ERR_ARG, "NULL preconditioner");
  if (nparams) *nparams = pc->nparam;
  if (block_sites) *block_sites = pc->per;
  if (npairs) *npairs = pc->npairs;
  return QED3_OK;
}

int qed3_lpc_get_weights(const qed3_lpc* pc, double* w) {
  QED3_GUARD_BEGIN
  if (!pc || !w) return fail(QED3_ERR_ARG, "NULL argument");
  return lpc_get_weights(pc, w);
  QED3_GUARD_END
}

int qed3_lpc_set_weights(qed3_lpc* pc, const double* w) {
  QED3_GUARD_BEGIN
  if (!pc || !w) return fail(QED3_ERR_ARG, "NULL argument");
  return lpc_set_weights(pc, w);
  QED3_GUARD_END
}

int qed3_lpc_apply(qed3_lpc* pc, int form, double* z, const double* r, int nrhs, void* stream) {
  QED3_GUARD_BEGIN
  if (!pc || !z || !r) return fail(QED3_ERR_ARG, "NULL argument");
  if (form != 0 && form != 1) return fail(QED3_ERR_ARG, "form must be 0 (layers) or 1 (words)");
  if (nrhs < 1) return fail(QED3_ERR_ARG, "nrhs must be positive");
  if (form == 1 && pc->C < (pc->LG == 2 ? 7 : 3)) return fail(QED3_ERR_ARG, "word form needs >= 7 (3) channels");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = size_t(nrhs) * pc->Ns * 2;
  float2 *fr = nullptr, *fz = nullptr;
  QED3_CUDA_TRY(cudaMalloc(&fr, n * sizeof(float2)));
  if (cudaMalloc(&fz, n * sizeof(float2)) != cudaSuccess) {
    cudaFree(fr);
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  int rc = field_import(pc->d, QED3_PREC_F32, fr, r, nrhs, st);
  if (!rc) rc = form == 0 ? lpc_forward(pc, nrhs, fr, fz, st) : lpc_apply_words(pc, nrhs, fr, fz, st);
  if (!rc) rc = field_export(pc->d, QED3_PREC_F32, z, fz, nrhs, st);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = fail(QED3_ERR_CUDA, "stream synchronize failed");
  cudaFree(fr);
  cudaFree(fz);
  return rc;
  QED3_GUARD_END
}

int qed3_lpc_loss_grad(qed3_lpc* pc, const double* r, const double* e, int nrhs, double* loss, double* grad,
                       void* stream) {
  QED3_GUARD_BEGIN
  if (!pc || !r || !e || !loss) return fail(QED3_ERR_ARG, "NULL argument");
  if (nrhs < 1) return fail(QED3_ERR_ARG, "nrhs must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = size_t(nrhs) * pc->Ns * 2;
  float2 *fr = nullptr, *fe = nullptr;
  QED3_CUDA_TRY(cudaMalloc(&fr, n * sizeof(float2)));
  if (cudaMalloc(&fe, n * sizeof(float2)) != cudaSuccess) {
    cudaFree(fr);
    return fail(QED3_ERR_NOMEM, "cudaMalloc failed");
  }
  int rc = field_import(pc->d, QED3_PREC_F32, fr, r, nrhs, st);
  if (!rc) rc = field_import(pc->d, QED3_PREC_F32, fe, e, nrhs, st);
  if (!rc) rc = lpc_loss_grad(pc, nrhs, fr, fe, loss, st);
  if (!rc && grad) {
    std::vector<float2> g(pc->nparam);
    if (cudaMemcpyAsync(g.data(), pc->G, pc->nparam * sizeof(float2), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = fail(QED3_ERR_CUDA, "gradient read-back failed");
    for (int i = 0; !rc && i < pc->nparam; i++) {
      grad[2 * i] = g[i].x;
      grad[2 * i + 1] = g[i].y;
    }
  }
  cudaFree(fr);
  cudaFree(fe);
  return rc;
  QED3_GUARD_END
}

int qed3_lpc_collect(qed3_lpc* pc, qed3_dirac* d, int nsrc, unsigned seed, const int* snapshots, int nsnap,
                     int precision) {
  QED3_GUARD_BEGIN
  if (!pc || !d || !snapshots) return fail(QED3_ERR_ARG, "NULL argument");
  if (nsrc < 1 || nsnap < 1) return fail(QED3_ERR_ARG, "nsrc and nsnap must be positive");
  if (precision < 0 || precision > 2) return fail(QED3_ERR_ARG, "unknown precision");
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set");
  return lpc_collect(pc, d, nsrc, seed, snapshots, nsnap, precision);
  QED3_GUARD_END
}

int qed3_lpc_train(qed3_lpc* pc, int steps, int batch, double lr, unsigned seed, double* loss_history) {
  QED3_GUARD_BEGIN
  if (!pc) return fail(QED3_ERR_ARG, "NULL preconditioner");
  if (steps < 0 || batch < 1 || !(lr > 0)) return fail(QED3_ERR_ARG, "need steps >= 0, batch >= 1, lr > 0");
  return lpc_train(pc, steps, batch, lr, seed, loss_history);
  QED3_GUARD_END
}

int qed3_lpc_set_tensor_cores(qed3_lpc* pc, int enable) {
  if (!pc) return fail(QED3_ERR_ARG, "NULL preconditioner");
  return lpc_set_tensor_cores(pc, enable);
}

int qed3_pcg_solve(qed3_dirac* d, qed3_lpc* pc, double* x, const double* b, const qed3_solve_params* params,
                   qed3_solve_report* report, void* stream) {
  QED3_GUARD_BEGIN
  if (!d || !pc || !x || !b) return fail(QED3_ERR_ARG, "NULL argument");
  return pcg_solve(d, pc, x, b, params, report, (cudaStream_t)stream);
  QED3_GUARD_END
}

}  // extern "C"
