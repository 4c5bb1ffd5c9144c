// Internal declarations shared by the qed3-gb300 translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/qed3.h"

namespace qed3 {

// ---------------------------------------------------------------------------
// Error plumbing: no exception crosses the C ABI.  Every entry point returns a
// status; the message of the last failure on the calling thread is kept for
// qed3_last_error_string().
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int selftest_wait_timeout(long long spin_limit, int* timed_out_v2, int* timed_out_streaming);

// ---------------------------------------------------------------------------
// Host lattice: the dual trivalent lattice S2Trivalent of the reference
// (src/both_3d/s2n_dual.h:15-173) built in O(N) from the icosahedral
// refinement, with the spin connection (omega, alpha) in closed form.
// All tables are in REFERENCE order (site = simplicial triangle id).
// ---------------------------------------------------------------------------
struct HostLattice {
  int n = 0;
  int n_sites = 0, n_links = 0, n_faces = 0;
  std::vector<double> simp_sites;    // [Nv*3]
  std::vector<int32_t> simp_faces;   // [Ns*3]
  std::vector<double> sites;         // [Ns*3]
  std::vector<int32_t> nns;          // [Ns*3], ascending
  std::vector<int32_t> links;        // [Nl*2], oriented links[l][0] -> links[l][1]; (i<j) lexicographic unless a caller's order was given
  std::vector<int32_t> simp_links;   // [Nl*2], (min,max)
  std::vector<int32_t> face_offsets; // [Nf+1]
  std::vector<int32_t> face_sites;   // ring of each dual face
  std::vector<double> ell, link_volume, vols;
  std::vector<double> tri_area;      // [Ns] spherical area of the triangle of dual site t (S2Simp::vols)
  double mean_ell = 0, mean_link_volume = 0, mean_vol = 0;
  std::vector<double> omega;         // [Nl], omega(links[l][0], links[l][1])
  std::vector<double> alpha;         // [Ns*3], alpha(x, nns[x][k])
  std::vector<int32_t> hop_link;     // [Ns*3]
  std::vector<int8_t> hop_sign;      // [Ns*3], +1 if the hop x -> y runs along its link's orientation
  std::vector<int8_t> hop_back;      // [Ns*3], slot of x in nns[y]
  std::vector<int32_t> face_links;   // [face_total], link id of (f[i], f[i+1])
  std::vector<int8_t> face_link_sign;// [face_total], +1 if f[i] -> f[i+1] runs along the link's orientation
  // space-filling-curve order used on the device
  std::vector<int32_t> perm;         // internal -> reference
  std::vector<int32_t> iperm;        // reference -> internal
};

int build_lattice(int n, bool sfc_order, HostLattice& L);
// the dual lattice of a caller's closed triangulation of the sphere; links:
// optional [Nl][2] link order (NULL = lexicographic)
int build_lattice_from_mesh(int n_vertices, const double* vertices, int n_triangles, const int32_t* triangles,
                            const int32_t* links, bool sfc_order, HostLattice& L);

// Zolotarev optimal rational approximation of sign(x) on [k, 1].
struct ZoloCoeffs {
  int n = 0, size = 0;
  double k = 0;
  std::vector<double> c, cp, A;
  double M = 0, lambda_inv = 0, E = 0, C = 0;
};
int zolotarev_coeffs(double k, int n, ZoloCoeffs& z);

}  // namespace qed3
