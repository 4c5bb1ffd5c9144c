// Builds the reference's own gauge field, Wilson action and force, and
// pure-gauge HMC (U1onS2, src/both/gauge.h; U1Wilson, src/both/action.h;
// HMCPureGauge, src/both/hmc.h:115-200; ParallelRng2, src/both/rng.h) from the
// reference tree, in place, into oracle/_ref/libgauge_ref.so.  Test
// infrastructure only: it pins the oracle's restatement of those pieces.  The
// templates take their lattice as a parameter; the lattice below carries the
// oracle's tables (faces as oriented site cycles, dual-face areas, links with
// their orientation) in the members those templates read.  The CUDA names are
// declared only so that the (never instantiated) fermion HMC templates in the
// same header parse; nothing here is copied from the reference.
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <iostream>
#include <map>
#include <random>
#include <string>
#include <vector>

#include <cuComplex.h>
#include <cuda_runtime.h>

using Idx = std::int32_t;
using CuC = cuDoubleComplex;
namespace Comp {
constexpr Idx N = 2;
}
#define CUDA_CHECK(x) (void)(x)
#define CD (sizeof(cuDoubleComplex))
#define D2D (cudaMemcpyDeviceToDevice)

#include REF_RNG_H
#include REF_GAUGE_H
#include REF_ACTION_H
#include REF_HMC_H

namespace {
struct TableLattice {
  using Link = std::array<int, 2>;
  int n_links = 0, n_sites = 0, n_faces = 0;
  std::vector<std::vector<int>> faces;
  std::vector<double> vols;
  double mean_vol = 0;
  std::map<Link, int> map2il, map2sign;
};

template <bool C>
void run(TableLattice& lat, double beta, const double* A, double* theta, double* avg, double* S, double* F, int seed,
         double tmax, int nsteps, int ntraj, double* A_out, double* dH, int* acc) {
  using Gauge = U1onS2<TableLattice, C>;
  Gauge U(lat);
  for (int l = 0; l < lat.n_links; l++) U[l] = A[l];
  for (int f = 0; f < lat.n_faces; f++) theta[f] = U.plaquette_angle(f);
  *avg = U.average_plaquette();
  U1Wilson SW(beta);
  *S = SW(U);
  Gauge dS(lat);
  SW.get_force(dS, U);
  for (int l = 0; l < lat.n_links; l++) F[l] = dS[l];
  ParallelRng2<TableLattice> rng(lat, seed);
  Gauge pi(lat);
  HMCPureGauge<ParallelRng2<TableLattice>, U1Wilson, Gauge, Gauge> hmc(rng, &SW, U, pi, tmax, nsteps);
  for (int t = 0; t < ntraj; t++) {
    double r = 0, d = 0;
    bool a = false;
    hmc.run(r, d, a);
    dH[t] = d;
    acc[t] = a ? 1 : 0;
  }
  for (int l = 0; l < lat.n_links; l++) A_out[l] = U[l];
}
}  // namespace

extern "C" void ref_gauge_run(int n_sites, int n_links, int n_faces, const int* face_off, const int* face_sites,
                              const double* vols, double mean_vol, const int* links, int compact, double beta,
                              const double* A, double* theta, double* avg, double* S, double* F, int seed,
                              double tmax, int nsteps, int ntraj, double* A_out, double* dH, int* acc) {
  TableLattice lat;
  lat.n_sites = n_sites;
  lat.n_links = n_links;
  lat.n_faces = n_faces;
  lat.mean_vol = mean_vol;
  lat.vols.assign(vols, vols + n_faces);
  for (int f = 0; f < n_faces; f++) lat.faces.emplace_back(face_sites + face_off[f], face_sites + face_off[f + 1]);
  for (int l = 0; l < n_links; l++) {
    const int x = links[2 * l], y = links[2 * l + 1];
    lat.map2il[{x, y}] = l;
    lat.map2il[{y, x}] = l;
    lat.map2sign[{x, y}] = 1;
    lat.map2sign[{y, x}] = -1;
  }
  if (compact)
    run<true>(lat, beta, A, theta, avg, S, F, seed, tmax, nsteps, ntraj, A_out, dH, acc);
  else
    run<false>(lat, beta, A, theta, avg, S, F, seed, tmax, nsteps, ntraj, A_out, dH, acc);
}
