// Builds the reference's own per-link / per-site random streams
// (ParallelRng2, src/both/rng.h:76-125, the engine ParallelRngExt uses per
// time slice in src/both_3d/rng.h) from the reference tree, in place, into
// oracle/_ref/librng_ref.so.  Test infrastructure only: it pins the oracle's
// RNG restatement.  Only the lattice type the template asks for is defined
// here; nothing is copied from the reference.
#include <cstdint>
#include <random>
#include <vector>

using Idx = std::int32_t;
#include REF_RNG_H

namespace {
struct SizesOnly {
  int n_links, n_sites;
};
}  // namespace

// Draws, in this order: two sweeps of gaussian_link over all links; per site
// the four gaussian_site values fill_gaussian takes (re, im for each spin);
// five master uniforms; per site four z2_site values.
extern "C" void ref_rng_streams(int n_links, int n_sites, int seed, double* links2, double* sites4, double* unif5,
                                double* z2_4) {
  const SizesOnly lat{n_links, n_sites};
  ParallelRng2<SizesOnly> rng(lat, seed);
  for (int s = 0; s < 2; s++)
    for (int l = 0; l < n_links; l++) links2[s * n_links + l] = rng.gaussian_link(l);
  for (int x = 0; x < n_sites; x++)
    for (int k = 0; k < 4; k++) sites4[4 * x + k] = rng.gaussian_site(x);
  for (int k = 0; k < 5; k++) unif5[k] = rng.uniform();
  for (int x = 0; x < n_sites; x++)
    for (int k = 0; k < 4; k++) z2_4[4 * x + k] = rng.z2_site(x);
}
