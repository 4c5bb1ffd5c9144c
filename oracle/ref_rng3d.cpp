// Builds the reference's per-time-slice random streams with their checkpoint
// writer (ParallelRngExt<Lattice, Nt>::ckpoint, src/both_3d/rng.h:90-168) from
// the reference tree, in place, into oracle/_ref/librng3d_ref.so.  Test
// infrastructure only: it pins the library's checkpoint format.  Only the
// names the header's (unused) fill_gaussian member refers to are declared
// here; nothing is copied from the reference.
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

using Idx = std::int32_t;
using Complex = std::complex<double>;
static const Complex I(0.0, 1.0);
namespace Comp {
constexpr int Nt = 1;
constexpr Idx N_SITES = 1;
constexpr int NS = 2;
constexpr Idx Nx = 2;
}  // namespace Comp
using namespace Comp;

#include REF_RNG3D_H

namespace {
struct SizesOnly {
  int n_links, n_sites;
};
template <class R>
void draws(R& rng, int nl, int ns, int nu, bool z2, double* out) {
  int k = 0;
  for (int l = 0; l < nl; l++) out[k++] = rng.gaussian_link(0, l);
  for (int x = 0; x < ns; x++)
    for (int a = 0; a < 4; a++) out[k++] = rng.gaussian_site(0, x);
  for (int u = 0; u < nu; u++) out[k++] = rng.uniform();
  if (z2)
    for (int x = 0; x < ns; x++)
      for (int a = 0; a < 4; a++) out[k++] = rng.z2_site(0, x);
}
}  // namespace

// seed -> one sweep of link and site Gaussians and 3 master uniforms ->
// ckpoint(save_path) -> continuation (links, site Gaussians, 2 uniforms, Z2)
// into cont[].  If load_path is given, a fresh object reads it and its
// continuation goes to cont_loaded[].
extern "C" void ref_rng3d_run(int n_links, int n_sites, int seed, const char* save_path, const char* load_path,
                              double* cont, double* cont_loaded) {
  const SizesOnly lat{n_links, n_sites};
  std::vector<double> first(size_t(n_links) + 4 * size_t(n_sites) + 3);
  ParallelRngExt<SizesOnly, 1> rng(lat, seed);
  draws(rng, n_links, n_sites, 3, false, first.data());
  if (save_path) rng.ckpoint(save_path);
  draws(rng, n_links, n_sites, 2, true, cont);
  if (load_path) {
    ParallelRngExt<SizesOnly, 1> other(lat, seed + 1);
    other.read(load_path);
    draws(other, n_links, n_sites, 2, true, cont_loaded);
  }
}
