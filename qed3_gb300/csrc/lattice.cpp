// Dual trivalent lattice on the refined icosahedron, built in O(N).
//
// Counterpart of the reference's offline generator and loaders:
//   integrator/get_geometry.cc:68-339  (sites, dual links, faces)
//   integrator/test_sorting.cc:139-289 (spin connection omega, alpha)
//   src/both_3d/s2n_simp.h:366-402, src/both_3d/s2n_dual.h:109-166 (areas)
// The reference finds links with an O(N^2) distance threshold and integrates
// omega numerically along each geodesic; here links come from the refinement's
// combinatorics and omega from the closed form
//     int_x^y cos(theta) dphi = dphi - (signed area of triangle (pole, x, y)),
// evaluated about the nearer pole, which is exact for great-circle arcs.
// Vertex/triangle numbering is this project's fixed convention (the reference
// inherits it from the absent QFE library): poles + two rings of five, flat
// barycentric subdivision projected radially; vertices = 12 corners, then
// edge interiors, then face interiors; triangles face-major, i-major,
// up-triangle then down-triangle.
//
// Compiled with -ffp-contract=off so coordinates are bit-identical on x86-64
// and aarch64 hosts.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <numeric>
#include <string>
#include <utility>
#include <vector>

#include "qed3_internal.h"

namespace qed3 {
namespace {

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 unit(V3 p) { return (1.0 / std::sqrt(dot(p, p))) * p; }

// Spherical triangle area (L'Huilier), as src/both_3d/s2n_dual.h:124-131.
double sph_area(V3 x, V3 y, V3 p) {
  const double a = std::acos(dot(x, p) / (norm(x) * norm(p)));
  const double b = std::acos(dot(y, p) / (norm(y) * norm(p)));
  const double c = std::acos(dot(x, y) / (norm(x) * norm(y)));
  const double s = 0.5 * (a + b + c);
  const double t = std::tan(0.5 * s) * std::tan(0.5 * (s - a)) * std::tan(0.5 * (s - b)) * std::tan(0.5 * (s - c));
  return 4.0 * std::atan(std::sqrt(t));
}

// Circumcentre of three points, the formula of integrator/geodesic.h:72-83.
V3 circumcentre(V3 r0, V3 r1, V3 r2) {
  const V3 r10 = r1 - r0;
  const V3 r20 = r2 - r0;
  const V3 t = dot(r10, r10) * r20 - dot(r20, r20) * r10;
  const V3 cr = cross(r10, r20);
  const V3 num = cross(t, cr);
  const double den = 2.0 * dot(cr, cr);
  return (1.0 / den) * num + r0;
}

// Tangent angle (in the frame e_theta, e_phi at p) of the direction d.
double frame_angle(V3 p, V3 d) {
  const double rho = std::sqrt(p.x * p.x + p.y * p.y);
  const double cth = p.z, sth = rho;  // |p| = 1
  const double cph = p.x / rho, sph = p.y / rho;
  const V3 et{cth * cph, cth * sph, -sth};
  const V3 ep{-sph, cph, 0.0};
  return std::atan2(dot(d, ep), dot(d, et));
}

// int cos(theta) dphi along the short great-circle arc x -> y.
double spin_connection(V3 x, V3 y) {
  const double phx = std::atan2(x.y, x.x), phy = std::atan2(y.y, y.x);
  double dphi = phy - phx;
  if (dphi > M_PI) dphi -= 2.0 * M_PI;
  if (dphi < -M_PI) dphi += 2.0 * M_PI;
  const double trip = x.x * y.y - x.y * y.x;  // z-component of x cross y
  const double xy = dot(x, y);
  if (x.z + y.z >= 0.0) return dphi - 2.0 * std::atan2(trip, 1.0 + x.z + y.z + xy);
  return 2.0 * std::atan2(trip, 1.0 - x.z - y.z + xy) - dphi;
}

struct Icosa {
  std::array<V3, 12> v;
  std::array<std::array<int, 3>, 20> f;
};

Icosa icosahedron() {
  Icosa ic;
  const double zr = 1.0 / std::sqrt(5.0);
  const double rr = 2.0 / std::sqrt(5.0);
  ic.v[0] = {0.0, 0.0, 1.0};
  for (int k = 0; k < 5; k++) {
    const double p1 = 2.0 * M_PI * k / 5.0;
    const double p2 = p1 + M_PI / 5.0;
    ic.v[1 + k] = {rr * std::cos(p1), rr * std::sin(p1), zr};
    ic.v[6 + k] = {rr * std::cos(p2), rr * std::sin(p2), -zr};
  }
  ic.v[11] = {0.0, 0.0, -1.0};
  int nf = 0;
  for (int k = 0; k < 5; k++) ic.f[nf++] = {0, 1 + k, 1 + (k + 1) % 5};
  for (int k = 0; k < 5; k++) ic.f[nf++] = {1 + k, 6 + k, 1 + (k + 1) % 5};
  for (int k = 0; k < 5; k++) ic.f[nf++] = {1 + (k + 1) % 5, 6 + k, 6 + (k + 1) % 5};
  for (int k = 0; k < 5; k++) ic.f[nf++] = {11, 6 + (k + 1) % 5, 6 + k};
  for (auto& t : ic.f) {
    const V3 a = ic.v[t[0]], b = ic.v[t[1]], c = ic.v[t[2]];
    if (dot(cross(b - a, c - a), a + b + c) < 0.0) std::swap(t[1], t[2]);
  }
  return ic;
}

inline uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

}  // namespace

// Simplicial vertices and triangles of the n-fold refined icosahedron.
static int refine_icosahedron(int n, std::vector<V3>& vert, std::vector<int32_t>& tri) {
  const Icosa ic = icosahedron();
  const int64_t Nv = 10LL * n * n + 2, Ns = 20LL * n * n;

  // ---- simplicial vertices --------------------------------------------------
  vert.clear();
  vert.reserve(size_t(Nv));
  for (int i = 0; i < 12; i++) vert.push_back(ic.v[i]);
  std::vector<std::array<int, 2>> edges;
  for (auto& t : ic.f)
    for (int e = 0; e < 3; e++) {
      int a = t[e], b = t[(e + 1) % 3];
      if (a > b) std::swap(a, b);
      edges.push_back({a, b});
    }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  int edge_base[12][12];
  for (auto& e : edges) {
    edge_base[e[0]][e[1]] = int(vert.size());
    for (int t = 1; t < n; t++) vert.push_back(unit(double(n - t) * ic.v[e[0]] + double(t) * ic.v[e[1]]));
  }
  tri.clear();
  tri.reserve(size_t(Ns) * 3);
  for (int f = 0; f < 20; f++) {
    const int A = ic.f[f][0], B = ic.f[f][1], C = ic.f[f][2];
    const V3 a = ic.v[A], b = ic.v[B], c = ic.v[C];
    // interior (i >= 1, j >= 1, i + j <= n - 1), i-major
    std::vector<int32_t> rowbase(n + 1, 0);
    const int ibase = int(vert.size());
    int cnt = 0;
    for (int i = 1; i <= n - 2; i++) {
      rowbase[i] = cnt;
      for (int j = 1; j <= n - 1 - i; j++, cnt++)
        vert.push_back(unit(double(n - i - j) * a + double(i) * b + double(j) * c));
    }
    auto edge_pt = [&](int u, int v, int t) -> int32_t {
      if (t == 0) return u;
      if (t == n) return v;
      if (u < v) return edge_base[u][v] + (t - 1);
      return edge_base[v][u] + (n - t - 1);
    };
    auto P = [&](int i, int j) -> int32_t {
      if (i == 0 && j == 0) return A;
      if (j == 0) return edge_pt(A, B, i);
      if (i == 0) return edge_pt(A, C, j);
      if (i + j == n) return edge_pt(B, C, j);
      return ibase + rowbase[i] + (j - 1);
    };
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n - i; j++) {
        tri.insert(tri.end(), {P(i, j), P(i + 1, j), P(i, j + 1)});
        if (i + j <= n - 2) tri.insert(tri.end(), {P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)});
      }
  }
  if (int64_t(vert.size()) != Nv || int64_t(tri.size()) != 3 * Ns) return fail(QED3_ERR_STATE, "refinement count mismatch");
  return QED3_OK;
}

// The dual trivalent lattice of a closed triangulation of the sphere:
// dual site t = triangle t, dual links = shared edges, dual faces = vertex
// rings; lengths, areas, spin connection and the device order.  Checks that
// the mesh is a closed 2-manifold of genus 0.
static int build_dual(const std::vector<V3>& vert, const std::vector<int32_t>& tri, bool sfc_order, HostLattice& L) {
  const int64_t Nv = int64_t(vert.size()), Ns = int64_t(tri.size()) / 3, Nl = 3 * Ns / 2;
  if (Ns < 4 || 3 * Ns != int64_t(tri.size()) || Ns % 2) return fail(QED3_ERR_ARG, "mesh: bad triangle count");
  if (Nv - Nl + Ns != 2) return fail(QED3_ERR_ARG, "mesh: not a closed triangulation of the sphere (V - E + F != 2)");
  for (int64_t t = 0; t < Ns; t++) {
    const int32_t a = tri[3 * t], b = tri[3 * t + 1], c = tri[3 * t + 2];
    if (a < 0 || b < 0 || c < 0 || a >= Nv || b >= Nv || c >= Nv || a == b || b == c || a == c)
      return fail(QED3_ERR_ARG, "mesh: bad vertex index in triangle " + std::to_string(t));
  }
  L.n_sites = int(Ns);
  L.n_links = int(Nl);
  L.n_faces = int(Nv);
  L.simp_sites.resize(size_t(Nv) * 3);
  for (int64_t v = 0; v < Nv; v++) {
    L.simp_sites[3 * v] = vert[v].x;
    L.simp_sites[3 * v + 1] = vert[v].y;
    L.simp_sites[3 * v + 2] = vert[v].z;
  }
  L.simp_faces = tri;

  // ---- dual sites: normalised circumcentres ---------------------------------
  std::vector<V3> site(static_cast<size_t>(Ns));
  L.sites.resize(size_t(Ns) * 3);
  for (int64_t t = 0; t < Ns; t++) {
    const V3 p = circumcentre(vert[tri[3 * t]], vert[tri[3 * t + 1]], vert[tri[3 * t + 2]]);
    site[t] = (1.0 / norm(p)) * p;
    L.sites[3 * t] = site[t].x;
    L.sites[3 * t + 1] = site[t].y;
    L.sites[3 * t + 2] = site[t].z;
  }

  // ---- vertex -> incident triangles (ascending) ------------------------------
  std::vector<int32_t> inc_off(size_t(Nv) + 1, 0), inc(size_t(Ns) * 3);
  for (int64_t t = 0; t < 3 * Ns; t++) inc_off[tri[t] + 1]++;
  for (int64_t v = 0; v < Nv; v++) inc_off[v + 1] += inc_off[v];
  {
    std::vector<int32_t> pos(inc_off.begin(), inc_off.end() - 1);
    for (int64_t t = 0; t < Ns; t++)
      for (int k = 0; k < 3; k++) inc[pos[tri[3 * t + k]]++] = int32_t(t);
  }

  // ---- dual links: triangles sharing an edge ----------------------------------
  // For triangle t and its edge (u,v), the other triangle is the one incident
  // to both u and v.
  std::vector<std::array<int32_t, 4>> lk;  // (i, j, simp_min, simp_max)
  lk.reserve(size_t(Nl));
  L.nns.assign(size_t(Ns) * 3, -1);
  for (int64_t t = 0; t < Ns; t++) {
    int32_t nb[3];
    int cnt = 0;
    for (int e = 0; e < 3; e++) {
      const int32_t u = tri[3 * t + e], v = tri[3 * t + (e + 1) % 3];
      int32_t other = -1, found = 0;
      for (int32_t a = inc_off[u]; a < inc_off[u + 1]; a++) {
        const int32_t s = inc[a];
        if (s == t) continue;
        for (int32_t b = inc_off[v]; b < inc_off[v + 1]; b++)
          if (inc[b] == s) {
            other = s;
            found++;
          }
      }
      if (found != 1) return fail(QED3_ERR_ARG, "mesh: an edge is not shared by exactly two triangles");
      nb[cnt++] = other;
      if (t < other) lk.push_back({int32_t(t), other, std::min(u, v), std::max(u, v)});
    }
    std::sort(nb, nb + 3);
    for (int k = 0; k < 3; k++) L.nns[3 * t + k] = nb[k];
  }
  std::sort(lk.begin(), lk.end());
  if (int64_t(lk.size()) != Nl) return fail(QED3_ERR_ARG, "mesh: link count mismatch");
  for (int64_t x = 0; x < Ns; x++)
    if (L.nns[3 * x] == L.nns[3 * x + 1] || L.nns[3 * x + 1] == L.nns[3 * x + 2])
      return fail(QED3_ERR_ARG, "mesh: two triangles share more than one edge");
  L.links.resize(size_t(Nl) * 2);
  L.simp_links.resize(size_t(Nl) * 2);
  for (int64_t l = 0; l < Nl; l++) {
    L.links[2 * l] = lk[l][0];
    L.links[2 * l + 1] = lk[l][1];
    L.simp_links[2 * l] = lk[l][2];
    L.simp_links[2 * l + 1] = lk[l][3];
  }
  // hop -> link id: links are sorted, so (min, max) is found by bisection
  auto link_id = [&](int32_t a, int32_t b) -> int32_t {
    const int32_t i = std::min(a, b), j = std::max(a, b);
    int64_t lo = 0, hi = Nl - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      const int32_t mi = L.links[2 * mid], mj = L.links[2 * mid + 1];
      if (mi < i || (mi == i && mj < j)) lo = mid + 1;
      else hi = mid;
    }
    return (L.links[2 * lo] == i && L.links[2 * lo + 1] == j) ? int32_t(lo) : -1;
  };
  L.hop_link.resize(size_t(Ns) * 3);
  L.hop_sign.resize(size_t(Ns) * 3);
  L.hop_back.resize(size_t(Ns) * 3);
  for (int64_t x = 0; x < Ns; x++)
    for (int k = 0; k < 3; k++) {
      const int32_t y = L.nns[3 * x + k];
      L.hop_link[3 * x + k] = link_id(int32_t(x), y);
      L.hop_sign[3 * x + k] = x < y ? 1 : -1;
      int kb = 0;
      while (kb < 3 && L.nns[3 * y + kb] != x) kb++;
      if (kb == 3) return fail(QED3_ERR_STATE, "asymmetric neighbour table");
      L.hop_back[3 * x + k] = int8_t(kb);
    }

  // ---- dual faces: the oriented ring walk of integrator/get_geometry.cc:252-339
  L.face_offsets.assign(size_t(Nv) + 1, 0);
  L.face_sites.clear();
  L.face_sites.reserve(size_t(Ns) * 3);
  for (int64_t v = 0; v < Nv; v++) {
    const int32_t* ring = &inc[inc_off[v]];
    const int m = inc_off[v + 1] - inc_off[v];
    std::vector<std::array<int32_t, 2>> fl;
    for (int i = 0; i < m; i++)
      for (int j = i + 1; j < m; j++)
        if (link_id(ring[i], ring[j]) >= 0) fl.push_back({ring[i], ring[j]});
    size_t il = 0;
    const V3 x0 = vert[v];
    while (true) {
      const auto e = fl[il];
      fl.erase(fl.begin() + long(il));
      const V3 x1 = site[e[0]], x2 = site[e[1]];
      const bool neg = dot(cross(x1 - x0, x2 - x1), x0) < 0.0;
      const int32_t first = neg ? e[1] : e[0], next = neg ? e[0] : e[1];
      L.face_sites.push_back(first);
      if (fl.empty()) break;
      bool more = false;
      for (size_t jl = 0; jl < fl.size(); jl++)
        if (fl[jl][0] == next || fl[jl][1] == next) {
          il = jl;
          more = true;
        }
      if (!more) return fail(QED3_ERR_ARG, "mesh: the triangles around a vertex do not form one ring");
    }
    if (int32_t(L.face_sites.size()) - L.face_offsets[v] != m)
      return fail(QED3_ERR_ARG, "mesh: the triangles around a vertex do not form one ring");
    L.face_offsets[v + 1] = int32_t(L.face_sites.size());
  }
  L.face_links.resize(L.face_sites.size());
  L.face_link_sign.resize(L.face_sites.size());
  for (int64_t v = 0; v < Nv; v++) {
    const int32_t o = L.face_offsets[v], m = L.face_offsets[v + 1] - o;
    for (int i = 0; i < m; i++) {
      const int32_t a = L.face_sites[o + i], b = L.face_sites[o + (i + 1) % m];
      L.face_links[o + i] = link_id(a, b);
      L.face_link_sign[o + i] = a < b ? 1 : -1;
    }
  }

  // ---- lengths and areas ---------------------------------------------------------
  L.ell.resize(size_t(Nl));
  L.link_volume.resize(size_t(Nl));
  for (int64_t l = 0; l < Nl; l++) {
    const V3 x = site[L.links[2 * l]], y = site[L.links[2 * l + 1]];
    const V3 pA = vert[L.simp_links[2 * l]], pB = vert[L.simp_links[2 * l + 1]];
    L.ell[l] = std::acos(dot(x, y) / (norm(x) * norm(y)));
    L.link_volume[l] = sph_area(x, y, pA) + sph_area(x, y, pB);
  }
  double s = 0;
  for (double e : L.link_volume) s += e;
  L.mean_link_volume = s / double(Nl);
  s = 0;
  for (double e : L.ell) s += e;
  L.mean_ell = s / double(Nl);
  // area of each triangle = dual site, S2Simp::vols (src/both_3d/s2n_simp.h:234-253)
  L.tri_area.resize(size_t(Ns));
  for (int64_t t = 0; t < Ns; t++) {
    const V3 x0 = vert[tri[3 * t]], x1 = vert[tri[3 * t + 1]], x2 = vert[tri[3 * t + 2]];
    const double a_ = std::acos(dot(x0, x1)), b_ = std::acos(dot(x1, x2)), c_ = std::acos(dot(x2, x0));
    const double s_ = 0.5 * (a_ + b_ + c_);
    const double tt = std::tan(0.5 * s_) * std::tan(0.5 * (s_ - a_)) * std::tan(0.5 * (s_ - b_)) * std::tan(0.5 * (s_ - c_));
    L.tri_area[t] = 4.0 * std::atan(std::sqrt(tt));
  }
  L.vols.resize(size_t(Nv));
  for (int64_t v = 0; v < Nv; v++) {
    double area = 0;
    const int32_t o = L.face_offsets[v], m = L.face_offsets[v + 1] - o;
    for (int i = 0; i < m; i++)
      area += sph_area(site[L.face_sites[o + i]], site[L.face_sites[o + (i + 1) % m]], vert[v]);
    L.vols[v] = area;
  }
  s = 0;
  for (double e : L.vols) s += e;
  L.mean_vol = s / double(Nv);

  // ---- spin connection --------------------------------------------------------------
  // omega(i,j) for links (i<j) with the section cut at phi0 = pi/48
  // (integrator/test_sorting.cc:203-235); alpha(x,y) = angle of the geodesic
  // x -> y at x in (-pi, pi] for x<y and in [0, 2pi) for x>y, the ranges the
  // reference's tables carry (integrator/test_sorting.cc:240-289).
  // The reference's test |d1| + |d2| - |d| < 1e-6 (and its refusal of sites
  // within 1e-6 of the cut) is replaced by the exact side test: a link crosses
  // the cut when its endpoints lie on opposite sides of the half-meridian phi0
  // and its short arc passes through phi0 (not phi0 + pi).  Both agree when
  // no site is within 1e-6 of the cut; for n >= 256 some are, and the exact
  // test keeps every face consistent.
  const double phi0 = M_PI / 48.0;
  L.omega.resize(size_t(Nl));
  for (int64_t l = 0; l < Nl; l++) {
    const V3 x = site[L.links[2 * l]], y = site[L.links[2 * l + 1]];
    double om = spin_connection(x, y);
    auto wrap = [](double a) {
      if (a >= M_PI) a -= 2.0 * M_PI;
      else if (a < -M_PI) a += 2.0 * M_PI;
      return a;
    };
    const double p1 = std::atan2(x.y, x.x), p2 = std::atan2(y.y, y.x);
    const double d1 = wrap(p1 - phi0), d2 = wrap(p2 - phi0);
    const bool opposite = (d1 >= 0.0) != (d2 >= 0.0);
    if (opposite && std::abs(d1) + std::abs(d2) < M_PI) om -= 2.0 * M_PI;
    L.omega[l] = om;
  }
  L.alpha.resize(size_t(Ns) * 3);
  for (int64_t x = 0; x < Ns; x++)
    for (int k = 0; k < 3; k++) {
      const int32_t y = L.nns[3 * x + k];
      const V3 p = site[x], q = site[y];
      const V3 d = q - dot(p, q) * p;  // tangent of the geodesic p -> q at p
      double al;
      if (x < y) {
        al = frame_angle(p, d);
      } else {
        // end tangent of the geodesic q -> p (pointing away from q), turned
        // by pi and reduced to [0, 2pi) as integrator/test_sorting.cc:288
        const double a1 = frame_angle(p, -1.0 * d) + M_PI;
        al = a1 - std::floor(a1 / (2.0 * M_PI)) * (2.0 * M_PI);
      }
      L.alpha[3 * x + k] = al;
    }

  // ---- device order: Morton code of the unit vectors --------------------------
  L.perm.resize(size_t(Ns));
  L.iperm.resize(size_t(Ns));
  std::iota(L.perm.begin(), L.perm.end(), 0);
  if (sfc_order) {
    std::vector<uint64_t> key(static_cast<size_t>(Ns));
    const double q = double((1u << 21) - 1);
    for (int64_t t = 0; t < Ns; t++) {
      const uint64_t ix = uint64_t((site[t].x + 1.0) * 0.5 * q);
      const uint64_t iy = uint64_t((site[t].y + 1.0) * 0.5 * q);
      const uint64_t iz = uint64_t((site[t].z + 1.0) * 0.5 * q);
      key[t] = spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2);
    }
    std::stable_sort(L.perm.begin(), L.perm.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  }
  for (int64_t i = 0; i < Ns; i++) L.iperm[L.perm[i]] = int32_t(i);
  return QED3_OK;
}

// Renumbers and orients the links as a caller lists them (a permutation of
// the lattice's links, each (i, j) in either order): links[l][0] -> links[l][1]
// becomes the positive direction of link l (the reference's map2sign,
// src/both_3d/s2n_dual.h:94-101), so hop and face signs follow the stored
// orientation and omega of a reversed link changes sign (the same spin
// connection per hop).  Every link-indexed table follows.
static int reorder_links(const int32_t* order, HostLattice& L) {
  const int64_t Nl = L.n_links;
  std::map<std::pair<int32_t, int32_t>, int32_t> pos;
  for (int64_t l = 0; l < Nl; l++) pos[{L.links[2 * l], L.links[2 * l + 1]}] = int32_t(l);
  std::vector<int32_t> old_of(size_t(Nl), -1), new_of(size_t(Nl), -1);
  std::vector<char> flip(size_t(Nl), 0);
  for (int64_t u = 0; u < Nl; u++) {
    const int32_t i = std::min(order[2 * u], order[2 * u + 1]), j = std::max(order[2 * u], order[2 * u + 1]);
    flip[u] = order[2 * u] > order[2 * u + 1];
    const auto it = pos.find({i, j});
    if (it == pos.end()) return fail(QED3_ERR_ARG, "links: (" + std::to_string(i) + ", " + std::to_string(j) +
                                                       ") is not a link of the mesh");
    if (new_of[it->second] >= 0) return fail(QED3_ERR_ARG, "links: a link is listed twice");
    old_of[u] = it->second;
    new_of[it->second] = int32_t(u);
  }
  auto permute2 = [&](std::vector<int32_t>& v) {
    std::vector<int32_t> w(v.size());
    for (int64_t u = 0; u < Nl; u++) {
      w[2 * u] = v[2 * size_t(old_of[u])];
      w[2 * u + 1] = v[2 * size_t(old_of[u]) + 1];
    }
    v.swap(w);
  };
  auto permute1 = [&](std::vector<double>& v) {
    std::vector<double> w(v.size());
    for (int64_t u = 0; u < Nl; u++) w[u] = v[old_of[u]];
    v.swap(w);
  };
  permute2(L.links);
  permute2(L.simp_links);
  permute1(L.ell);
  permute1(L.link_volume);
  permute1(L.omega);
  for (int64_t u = 0; u < Nl; u++)
    if (flip[u]) {
      std::swap(L.links[2 * u], L.links[2 * u + 1]);
      L.omega[u] = -L.omega[u];
    }
  for (auto& h : L.hop_link) h = new_of[h];
  for (auto& h : L.face_links) h = new_of[h];
  const int64_t Ns = L.n_sites;
  for (int64_t x = 0; x < Ns; x++)
    for (int k = 0; k < 3; k++) L.hop_sign[3 * x + k] = L.links[2 * size_t(L.hop_link[3 * x + k])] == x ? 1 : -1;
  for (size_t e = 0; e < L.face_sites.size(); e++)
    L.face_link_sign[e] = L.links[2 * size_t(L.face_links[e])] == L.face_sites[e] ? 1 : -1;
  return QED3_OK;
}

int build_lattice(int n, bool sfc_order, HostLattice& L) {
  if (n < 1 || n > 2048) return fail(QED3_ERR_ARG, "n_refine must be in [1, 2048]");
  if (20LL * n * n > (1LL << 30)) return fail(QED3_ERR_ARG, "lattice too large for int32 tables");
  L = HostLattice{};
  std::vector<V3> vert;
  std::vector<int32_t> tri;
  int rc = refine_icosahedron(n, vert, tri);
  if (!rc) rc = build_dual(vert, tri, sfc_order, L);
  L.n = n;
  return rc;
}

int build_lattice_from_mesh(int n_vertices, const double* vertices, int n_triangles, const int32_t* triangles,
                            const int32_t* links, bool sfc_order, HostLattice& L) {
  if (n_vertices < 4 || n_triangles < 4 || int64_t(n_triangles) > (1LL << 30))
    return fail(QED3_ERR_ARG, "mesh: bad vertex or triangle count");
  L = HostLattice{};
  std::vector<V3> vert(static_cast<size_t>(n_vertices));
  for (int v = 0; v < n_vertices; v++) {
    const V3 p{vertices[3 * v], vertices[3 * v + 1], vertices[3 * v + 2]};
    const double r = norm(p);
    if (!(r > 0.0) || !std::isfinite(r)) return fail(QED3_ERR_ARG, "mesh: vertex " + std::to_string(v) + " is zero");
    // unit vectors (to rounding) are taken as given, so a mesh exported by
    // qed3_lattice_mesh rebuilds the identical lattice
    vert[v] = std::abs(r - 1.0) <= 4e-16 ? p : (1.0 / r) * p;
  }
  std::vector<int32_t> tri(triangles, triangles + 3 * size_t(n_triangles));
  int rc = build_dual(vert, tri, sfc_order, L);
  if (!rc && links) rc = reorder_links(links, L);
  L.n = 0;
  return rc;
}

}  // namespace qed3
