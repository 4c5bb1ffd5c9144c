// Persistent CG on D^dagger D (+ shift): one cooperative launch per solve.
//
// Replaces MatPoly::solve<N> (src/dual/matpoly.h:204-267), which per
// iteration launched two CSR SpMVs, three axpy kernels and two cuBLAS Zdotc
// calls that each returned to the host, plus two cudaMalloc/cudaFree and
// ~5 device copies (src/dual/matpoly.h:62-84).  Here the whole solve is one
// kernel: per iteration two phases, each a gather stencil with the CG vector
// updates and the dot product fused in, separated by a grid barrier whose
// arrival also publishes the block partial sums (FP64, summed in a fixed
// order by every block, so all blocks agree bit for bit).
//
//   phase A: t = a_r D r + beta t ; p = a_r r + beta p ; gamma = |t|^2 + s|p|^2
//            (t stays equal to D p without ever gathering p)
//   phase B: q = D^dag t + s p ; x += alpha p ; r -= alpha q ; mu = |r|^2
//
// Mixed precision (F32 / BF16 storage of the gathered fields): fp32 arithmetic,
// FP64 accumulation of every dot product, and a reliable update whenever
// |r| drops below delta * max|r| since the last one: x_hi += x_lo and
// r = b - A x_hi recomputed with the FP64 operator, p re-orthogonalised
// against the new r.  Convergence is decided ONLY on that FP64 true residual.
// Plain FP64 mode uses the same machinery with the true-residual check at the
// point where the recursive residual reaches the tolerance.

#include <cmath>
#include <string>

#include "device.cuh"
#include "dirac_impl.h"
#include "handles.h"
#include "solver_v2.h"

namespace qed3 {

struct CgArgs {
  int Ns;
  const int* nbr;
  const M64* H;
  const M64* Hd;
  const double* diag;
  const M32* H32;
  const M32* Hd32;
  const float* diag32;
  const S64* b;
  S64* xhi;
  S64* xhi2;
  S64* t64;
  void* r;
  void* p;
  void* t;
  void* xlo;
  void* rh;          // gathered copy of r (== r for fp32; bf16 copy for bf16)
  void* th;          // gathered copy of t
  double* partials;  // [2][gridDim][4]
  GridBar* bar;
  double* scal;      // [0] mu_true [1] bnorm2 [2] iters [3] reliable updates [4] status [5] x buffer (0/1)
  double tol2;
  double delta2;
  double shift;
  int maxiter;
  long long spin_limit;
};

// Sum NV partials over all blocks after a barrier; every block gets the same
// bits.  Valid in all threads on return.
template <int NV>
__device__ __forceinline__ void grid_total(const double* part, double (&out)[NV], double* sh) {
  if (threadIdx.x < 32) {
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = 0.0;
    for (int bI = threadIdx.x; bI < gridDim.x; bI += 32)
#pragma unroll
      for (int q = 0; q < NV; q++) acc[q] += __ldcg(part + size_t(bI) * 4 + q);
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = warp_sum(acc[q]);
    if (threadIdx.x == 0)
#pragma unroll
      for (int q = 0; q < NV; q++) sh[q] = acc[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; q++) out[q] = sh[q];
  __syncthreads();
}

template <int NV>
__device__ __forceinline__ void publish(double (&v)[NV], double* part, double* sh) {
  block_sum<NV>(v, sh);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) __stcg(part + size_t(blockIdx.x) * 4 + q, v[q]);
}

// Low-precision accessors for the mixed kernel.
template <int P>
struct Mix {
  using Lo = typename LoField<P>::T;
};

template <int P>
__global__ void __launch_bounds__(256) k_cg_persistent(CgArgs a) {
  __shared__ double sh[32 * 4];
  const int Ns = a.Ns;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  unsigned int gen = 0;
  int phase = 0;
  auto part = [&]() { return a.partials + size_t(phase & 1) * gridDim.x * 4; };
  const bool mixed = (P != P64);

  using Lo = typename Mix<P == P64 ? P32 : P>::Lo;
  S64* r64 = reinterpret_cast<S64*>(a.r);
  S64* p64 = reinterpret_cast<S64*>(a.p);
  S64* t64w = reinterpret_cast<S64*>(a.t);
  // mixed modes keep r and t in fp32; neighbours are read from rh / th,
  // which alias r / t in fp32 mode and are bf16 copies in bf16 mode
  float4* r32 = reinterpret_cast<float4*>(a.r);
  float4* t32 = reinterpret_cast<float4*>(a.t);
  Lo* rh = reinterpret_cast<Lo*>(a.rh);
  Lo* th = reinterpret_cast<Lo*>(a.th);
  float4* p32 = reinterpret_cast<float4*>(a.p);
  float4* xlo = reinterpret_cast<float4*>(a.xlo);
  S64* xa = a.xhi;
  S64* xb = a.xhi2;

  // ---- phase 0: x = 0, r = b, p = t = 0; |b|^2 --------------------------------------
  {
    double v[1] = {0.0};
    for (int i = tid; i < Ns; i += nth) {
      const Sp64 bi = ld64(a.b, i);
      v[0] += bi.s0.x * bi.s0.x + bi.s0.y * bi.s0.y + bi.s1.x * bi.s1.x + bi.s1.y * bi.s1.y;
      const Sp64 z{make_double2(0, 0), make_double2(0, 0)};
      st64(xa, i, z);
      if constexpr (!mixed) {
        st64(r64, i, bi);
        st64(p64, i, z);
        st64(t64w, i, z);
      } else {
        const Sp32 bl{make_float2(float(bi.s0.x), float(bi.s0.y)), make_float2(float(bi.s1.x), float(bi.s1.y))};
        const Sp32 zl{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        st32(r32, i, bl);
        st32(t32, i, zl);
        if constexpr (P == PBF16) {
          stbf(reinterpret_cast<uint2*>(rh), i, bl);
          stbf(reinterpret_cast<uint2*>(th), i, zl);
        }
        st32(p32, i, zl);
        st32(xlo, i, zl);
      }
    }
    publish<1>(v, part(), sh);
    if (!grid_sync(a.bar, gen, a.spin_limit)) goto timeout;
    double tot[1];
    grid_total<1>(part(), tot, sh);
    phase++;
    const double bnorm2 = tot[0];
    if (bnorm2 == 0.0) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.scal[0] = 0.0; a.scal[1] = 0.0; a.scal[2] = 0; a.scal[3] = 0; a.scal[4] = QED3_OK; a.scal[5] = 0;
      }
      return;
    }

    double mu = bnorm2, mu_max = bnorm2, beta = 0.0;
    double2 a_r = make_double2(1.0, 0.0);
    int iter = 0, nru = 0, status = QED3_ERR_NOCONV;
    double mu_true = bnorm2;
    const double s = a.shift;

    while (true) {
      // ---- phase A ------------------------------------------------------------------
      {
        double v[1] = {0.0};
        for (int i = tid; i < Ns; i += nth) {
          if constexpr (!mixed) {
            const Sp64 dr = hop64(i, Ns, a.nbr, a.H, a.diag, r64);
            const Sp64 ti = ld64(t64w, i), pi = ld64(p64, i), ri = ld64(r64, i);
            Sp64 tn, pn;
            tn.s0 = cfma(a_r, dr.s0, cscale(beta, ti.s0));
            tn.s1 = cfma(a_r, dr.s1, cscale(beta, ti.s1));
            pn.s0 = cfma(a_r, ri.s0, cscale(beta, pi.s0));
            pn.s1 = cfma(a_r, ri.s1, cscale(beta, pi.s1));
            st64(t64w, i, tn);
            st64(p64, i, pn);
            v[0] += tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y +
                    s * (pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y);
          } else {
            const Sp32 ri = ld32(r32, i);
            const Sp32 dr = hop32_self<P>(i, Ns, a.nbr, a.H32, a.diag32, ri, rh);
            const Sp32 ti = ld32(t32, i), pi = ld32(p32, i);
            const float2 ar = make_float2(float(a_r.x), float(a_r.y));
            const float bt = float(beta);
            Sp32 tn, pn;
            tn.s0 = cfmaf(ar, dr.s0, make_float2(bt * ti.s0.x, bt * ti.s0.y));
            tn.s1 = cfmaf(ar, dr.s1, make_float2(bt * ti.s1.x, bt * ti.s1.y));
            pn.s0 = cfmaf(ar, ri.s0, make_float2(bt * pi.s0.x, bt * pi.s0.y));
            pn.s1 = cfmaf(ar, ri.s1, make_float2(bt * pi.s1.x, bt * pi.s1.y));
            st32(t32, i, tn);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(th), i, tn);
            st32(p32, i, pn);
            const float tt = tn.s0.x * tn.s0.x + tn.s0.y * tn.s0.y + tn.s1.x * tn.s1.x + tn.s1.y * tn.s1.y;
            const float pp = pn.s0.x * pn.s0.x + pn.s0.y * pn.s0.y + pn.s1.x * pn.s1.x + pn.s1.y * pn.s1.y;
            v[0] += double(tt) + s * double(pp);
          }
        }
        publish<1>(v, part(), sh);
        if (!grid_sync(a.bar, gen, a.spin_limit)) goto timeout;
      }
      double gam[1];
      grid_total<1>(part(), gam, sh);
      phase++;
      const double alpha = mu / gam[0];

      // ---- phase B ------------------------------------------------------------------
      {
        double v[1] = {0.0};
        for (int i = tid; i < Ns; i += nth) {
          if constexpr (!mixed) {
            const Sp64 q = hop64(i, Ns, a.nbr, a.Hd, a.diag, t64w);
            const Sp64 pi = ld64(p64, i), ri = ld64(r64, i), xi = ld64(xa, i);
            Sp64 rn, xn;
            rn.s0 = csub(ri.s0, cscale(alpha, cadd(q.s0, cscale(s, pi.s0))));
            rn.s1 = csub(ri.s1, cscale(alpha, cadd(q.s1, cscale(s, pi.s1))));
            xn.s0 = cadd(xi.s0, cscale(alpha, pi.s0));
            xn.s1 = cadd(xi.s1, cscale(alpha, pi.s1));
            st64(r64, i, rn);
            st64(xa, i, xn);
            v[0] += rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y;
          } else {
            const Sp32 ti = ld32(t32, i);
            const Sp32 q = hop32_self<P>(i, Ns, a.nbr, a.Hd32, a.diag32, ti, th);
            const Sp32 pi = ld32(p32, i), ri = ld32(r32, i), xi = ld32(xlo, i);
            const float al = float(alpha), sf = float(s);
            Sp32 rn, xn;
            rn.s0 = make_float2(ri.s0.x - al * (q.s0.x + sf * pi.s0.x), ri.s0.y - al * (q.s0.y + sf * pi.s0.y));
            rn.s1 = make_float2(ri.s1.x - al * (q.s1.x + sf * pi.s1.x), ri.s1.y - al * (q.s1.y + sf * pi.s1.y));
            xn.s0 = make_float2(xi.s0.x + al * pi.s0.x, xi.s0.y + al * pi.s0.y);
            xn.s1 = make_float2(xi.s1.x + al * pi.s1.x, xi.s1.y + al * pi.s1.y);
            st32(r32, i, rn);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(rh), i, rn);
            st32(xlo, i, xn);
            v[0] += double(rn.s0.x * rn.s0.x + rn.s0.y * rn.s0.y + rn.s1.x * rn.s1.x + rn.s1.y * rn.s1.y);
          }
        }
        publish<1>(v, part(), sh);
        if (!grid_sync(a.bar, gen, a.spin_limit)) goto timeout;
      }
      double mun[1];
      grid_total<1>(part(), mun, sh);
      phase++;
      iter++;
      const double mu_new = mun[0];
      const bool finite = isfinite(mu_new) && isfinite(alpha);
      mu_max = fmax(mu_max, mu_new);
      const bool want_check = !finite || mu_new < a.tol2 * bnorm2 || iter >= a.maxiter ||
                              (mixed && mu_new < a.delta2 * mu_max);
      if (!want_check) {
        beta = mu_new / mu;
        a_r = make_double2(1.0, 0.0);
        mu = mu_new;
        continue;
      }

      // ---- reliable update / true residual: R1  t64 = D (x_hi + x_lo), x_hi2 = x_hi + x_lo
      for (int i = tid; i < Ns; i += nth) {
        Sp64 o;
        if constexpr (!mixed) {
          o = hop64(i, Ns, a.nbr, a.H, a.diag, xa);
        } else {
          const int j[3] = {__ldg(a.nbr + i), __ldg(a.nbr + Ns + i), __ldg(a.nbr + 2 * Ns + i)};
          auto xs = [&](int k) {
            const Sp64 h = ld64(xa, k);
            const Sp32 l = ld32(xlo, k);
            return Sp64{make_double2(h.s0.x + l.s0.x, h.s0.y + l.s0.y), make_double2(h.s1.x + l.s1.x, h.s1.y + l.s1.y)};
          };
          const Sp64 self = xs(i);
          st64(xb, i, self);
          const double dg = __ldg(a.diag + i);
          o = Sp64{cscale(dg, self.s0), cscale(dg, self.s1)};
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const Sp64 bj = xs(j[k]);
            const M64 m = a.H[k * Ns + i];
            o.s0 = cfma(m.h00, bj.s0, o.s0);
            o.s0 = cfma(m.h01, bj.s1, o.s0);
            o.s1 = cfma(m.h10, bj.s0, o.s1);
            o.s1 = cfma(m.h11, bj.s1, o.s1);
          }
        }
        st64(a.t64, i, o);
      }
      if (!grid_sync(a.bar, gen, a.spin_limit)) goto timeout;
      if constexpr (mixed) {
        S64* tmp = xa;
        xa = xb;
        xb = tmp;
      }
      // ---- R2  r_true = b - D^dag t64 - s x ; |r_true|^2 and <r_true, p>
      {
        double v[3] = {0.0, 0.0, 0.0};
        for (int i = tid; i < Ns; i += nth) {
          const Sp64 q = hop64(i, Ns, a.nbr, a.Hd, a.diag, a.t64);
          const Sp64 bi = ld64(a.b, i), xi = ld64(xa, i);
          Sp64 rt;
          rt.s0 = csub(bi.s0, cadd(q.s0, cscale(s, xi.s0)));
          rt.s1 = csub(bi.s1, cadd(q.s1, cscale(s, xi.s1)));
          v[0] += rt.s0.x * rt.s0.x + rt.s0.y * rt.s0.y + rt.s1.x * rt.s1.x + rt.s1.y * rt.s1.y;
          double2 pv0, pv1;
          if constexpr (!mixed) {
            const Sp64 pi = ld64(p64, i);
            pv0 = pi.s0;
            pv1 = pi.s1;
            st64(r64, i, rt);
          } else {
            const Sp32 pi = ld32(p32, i);
            pv0 = make_double2(pi.s0.x, pi.s0.y);
            pv1 = make_double2(pi.s1.x, pi.s1.y);
            const Sp32 rl{make_float2(float(rt.s0.x), float(rt.s0.y)), make_float2(float(rt.s1.x), float(rt.s1.y))};
            st32(r32, i, rl);
            if constexpr (P == PBF16) stbf(reinterpret_cast<uint2*>(rh), i, rl);
            st32(xlo, i, Sp32{make_float2(0.f, 0.f), make_float2(0.f, 0.f)});
          }
          // <r, p> = sum conj(r) p
          v[1] += rt.s0.x * pv0.x + rt.s0.y * pv0.y + rt.s1.x * pv1.x + rt.s1.y * pv1.y;
          v[2] += rt.s0.x * pv0.y - rt.s0.y * pv0.x + rt.s1.x * pv1.y - rt.s1.y * pv1.x;
        }
        publish<3>(v, part(), sh);
        if (!grid_sync(a.bar, gen, a.spin_limit)) goto timeout;
      }
      double tr[3];
      grid_total<3>(part(), tr, sh);
      phase++;
      nru++;
      mu_true = tr[0];
      if (mu_true < a.tol2 * bnorm2) {
        status = QED3_OK;
        break;
      }
      if (iter >= a.maxiter || !isfinite(mu_true)) {
        status = QED3_ERR_NOCONV;
        break;
      }
      // continue: beta = |r_true|^2 / mu_old, p <- p - c r_true with c = <r,p>/|r|^2,
      // folded into the next phase A as p = (1 - beta c) r + beta p
      beta = mu_true / mu;
      a_r = make_double2(1.0 - beta * tr[1] / mu_true, -beta * tr[2] / mu_true);
      mu = mu_true;
      mu_max = mu_true;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.scal[0] = mu_true;
      a.scal[1] = bnorm2;
      a.scal[2] = iter;
      a.scal[3] = nru;
      a.scal[4] = status;
      a.scal[5] = (xa == a.xhi) ? 0 : 1;
    }
    return;
  }
timeout:
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[4] = QED3_ERR_TIMEOUT;
    a.scal[5] = 0;
  }
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
int cg_finish(qed3_dirac_s* d, double* x, qed3_solve_report* rep, cudaStream_t st);

int ensure_work(qed3_dirac_s* d) {
  SolverWork& w = d->work;
  const size_t Ns = size_t(d->Ns);
  if (w.ns == Ns) return QED3_OK;
  if (w.ns) solver_free(d);
  const size_t b64 = Ns * sizeof(S64);
  QED3_CUDA_TRY(cudaMalloc(&w.b, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.xhi, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.xhi2, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.rhi, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.t64, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.r, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.p, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.t, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.xlo, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.rg, b64));
  QED3_CUDA_TRY(cudaMalloc(&w.tg, b64));
  int dev = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  QED3_CUDA_TRY(cudaDeviceGetAttribute(&d->sm_count, cudaDevAttrMultiProcessorCount, dev));
  const size_t maxblocks = size_t(d->sm_count) * 32;
  QED3_CUDA_TRY(cudaMalloc(&w.partials, 2 * maxblocks * 4 * sizeof(double)));
  QED3_CUDA_TRY(cudaMalloc(&w.bar, sizeof(GridBar)));
  QED3_CUDA_TRY(cudaMalloc(&w.bar2, sizeof(GridBar2)));
  QED3_CUDA_TRY(cudaMalloc(&w.scal, 8 * sizeof(double)));
  QED3_CUDA_TRY(cudaEventCreate(&w.e0));
  QED3_CUDA_TRY(cudaEventCreate(&w.e1));
  w.ns = Ns;
  return QED3_OK;
}

int solver_free(qed3_dirac_s* d) {
  SolverWork& w = d->work;
  void* ptrs[] = {w.b, w.xhi, w.xhi2, w.rhi, w.t64, w.r, w.p, w.t, w.xlo, w.rg, w.tg, w.partials, w.bar, w.bar2, w.scal};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (w.e0) cudaEventDestroy(w.e0);
  if (w.e1) cudaEventDestroy(w.e1);
  w = SolverWork{};
  return QED3_OK;
}

template <int P>
static int launch_cg(qed3_dirac_s* d, CgArgs& args, cudaStream_t st) {
  int per_sm = 0;
  QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent<P>, 256, 0));
  if (per_sm < 1) return fail(QED3_ERR_CUDA, "persistent CG kernel cannot be resident");
  const long long need = (d->Ns + 255) / 256;
  long long grid = std::min<long long>(need, (long long)per_sm * d->sm_count);
  grid = std::min<long long>(grid, (long long)d->sm_count * 32);
  if (grid < 1) grid = 1;
  void* kargs[] = {&args};
  QED3_CUDA_TRY(cudaLaunchCooperativeKernel((void*)k_cg_persistent<P>, dim3(unsigned(grid)), dim3(256), kargs, 0, st));
  return QED3_OK;
}

// Launches the persistent CG kernel on caller-provided scratch (used by the
// allocation-free entry point); returns the grid size through *grid_out.
int cg_launch_on_scratch(int prec, qed3_dirac_s* d, S64* b, S64* xhi, S64* xhi2, S64* t64, void* r, void* p, void* t,
                         void* xlo, void* rh, void* th, double* partials, int max_blocks, GridBar* bar, double* scal,
                         double tol, double delta, int maxiter, double shift, cudaStream_t st) {
  int per_sm = 0, smc = 0, dev = 0;
  QED3_CUDA_TRY(cudaGetDevice(&dev));
  QED3_CUDA_TRY(cudaDeviceGetAttribute(&smc, cudaDevAttrMultiProcessorCount, dev));
  if (prec == QED3_PREC_F64)
    QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent<P64>, 256, 0));
  else if (prec == QED3_PREC_F32)
    QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent<P32>, 256, 0));
  else
    QED3_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent<PBF16>, 256, 0));
  if (per_sm < 1) return fail(QED3_ERR_CUDA, "persistent CG kernel cannot be resident");
  long long grid = std::min<long long>((d->Ns + 255) / 256, (long long)per_sm * smc);
  grid = std::max<long long>(1, std::min<long long>(grid, max_blocks));
  CgArgs a{};
  a.Ns = d->Ns;
  a.nbr = d->lat->dev.nbr;
  a.H = d->H;
  a.Hd = d->Hd;
  a.diag = d->diag;
  a.H32 = d->H32;
  a.Hd32 = d->Hd32;
  a.diag32 = d->diag32;
  a.b = b;
  a.xhi = xhi;
  a.xhi2 = xhi2;
  a.t64 = t64;
  a.r = r;
  a.p = p;
  a.t = t;
  a.xlo = xlo;
  a.rh = prec == QED3_PREC_BF16 ? rh : r;
  a.th = prec == QED3_PREC_BF16 ? th : t;
  a.partials = partials;
  a.bar = bar;
  a.scal = scal;
  a.tol2 = tol * tol;
  a.delta2 = delta * delta;
  a.shift = shift;
  a.maxiter = maxiter;
  a.spin_limit = 20000000LL;
  void* kargs[] = {&a};
  const void* fn = prec == QED3_PREC_F64   ? (const void*)k_cg_persistent<P64>
                   : prec == QED3_PREC_F32 ? (const void*)k_cg_persistent<P32>
                                           : (const void*)k_cg_persistent<PBF16>;
  QED3_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(unsigned(grid)), dim3(256), kargs, 0, st));
  return QED3_OK;
}

int cg_solve(qed3_dirac_s* d, double* x, const double* b, const qed3_solve_params* prm, qed3_solve_report* rep,
             cudaStream_t st) {
  if (!d->coeffs_set) return fail(QED3_ERR_STATE, "operator coefficients not set (call qed3_dirac_set_links)");
  int rc = ensure_work(d);
  if (rc) return rc;
  SolverWork& w = d->work;
  const int prec = prm ? prm->precision : QED3_PREC_F64;
  if (prec < QED3_PREC_F64 || prec > QED3_PREC_BF16) return fail(QED3_ERR_ARG, "unknown precision");
  const double tol = prm && prm->tol > 0 ? prm->tol : 1e-10;
  const double delta = prm && prm->delta > 0 ? prm->delta : 0.1;
  const int maxiter = prm && prm->maxiter > 0 ? prm->maxiter : 100000;
  const double shift = prm ? prm->shift : 0.0;

  rc = field_import_unit(d, w.b, b, w.partials, w.scal + 6, st);
  if (rc) return rc;
  // register-resident kernel when every site can own a thread
  int vgrid = 0, vthreads = 0, vspt = 0;
  const bool streaming = prm && (prm->flags & QED3_SOLVE_STREAMING);
  if (!streaming && cg_v2_plan(prec, d->Ns, d->sm_count, &vgrid, &vthreads, &vspt)) {
    QED3_CUDA_TRY(cudaMemsetAsync(w.bar2, 0, sizeof(GridBar2), st));
    CgV2Args v{};
    v.Ns = d->Ns;
    v.nbr = d->lat->dev.nbr;
    v.H = d->H;
    v.Hd = d->Hd;
    v.diag = d->diag;
    v.H32 = d->H32;
    v.Hd32 = d->Hd32;
    v.diag32 = d->diag32;
    v.b = w.b;
    v.x = w.xhi;
    v.t64 = w.t64;
    v.halo_r = w.r;
    v.halo_t = w.t;
    v.partials = w.partials;
    v.bar = w.bar2;
    v.scal = w.scal;
    v.tol2 = tol * tol;
    v.delta2 = delta * delta;
    v.shift = shift;
    v.maxiter = maxiter;
    v.spin_limit = 4000000LL;  // ~2-4 s of acquire polling before a barrier gives up
    QED3_CUDA_TRY(cudaEventRecord(w.e0, st));
    if ((rc = cg_v2_launch(prec, vspt, vgrid, vthreads, v, st))) return rc;
    QED3_CUDA_TRY(cudaEventRecord(w.e1, st));
    return cg_finish(d, x, rep, st);
  }
  QED3_CUDA_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBar), st));
  CgArgs a{};
  a.Ns = d->Ns;
  a.nbr = d->lat->dev.nbr;
  a.H = d->H;
  a.Hd = d->Hd;
  a.diag = d->diag;
  a.H32 = d->H32;
  a.Hd32 = d->Hd32;
  a.diag32 = d->diag32;
  a.b = w.b;
  a.xhi = w.xhi;
  a.xhi2 = w.xhi2;
  a.t64 = w.t64;
  a.r = w.r;
  a.p = w.p;
  a.t = w.t;
  a.xlo = w.xlo;
  a.rh = prec == QED3_PREC_BF16 ? w.rg : w.r;
  a.th = prec == QED3_PREC_BF16 ? w.tg : w.t;
  a.partials = w.partials;
  a.bar = w.bar;
  a.scal = w.scal;
  a.tol2 = tol * tol;
  a.delta2 = delta * delta;
  a.shift = shift;
  a.maxiter = maxiter;
  a.spin_limit = 20000000LL;  // ~1-2 s of polling before a barrier gives up
  QED3_CUDA_TRY(cudaEventRecord(w.e0, st));
  if (prec == QED3_PREC_F64) rc = launch_cg<P64>(d, a, st);
  else if (prec == QED3_PREC_F32) rc = launch_cg<P32>(d, a, st);
  else rc = launch_cg<PBF16>(d, a, st);
  if (rc) return rc;
  QED3_CUDA_TRY(cudaEventRecord(w.e1, st));
  return cg_finish(d, x, rep, st);
}

// Reads the device scalars, exports the solution buffer the kernel chose and
// fills the report.
int cg_finish(qed3_dirac_s* d, double* x, qed3_solve_report* rep, cudaStream_t st) {
  SolverWork& w = d->work;
  int rc;
  // export whichever x buffer holds the result (decided on the device)
  double sc[8];
  QED3_CUDA_TRY(cudaMemcpyAsync(sc, w.scal, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  QED3_CUDA_TRY(cudaStreamSynchronize(st));
  S64* xres = (sc[5] != 0.0) ? w.xhi2 : w.xhi;
  rc = field_export_scaled(d, x, xres, w.scal + 6, st);
  if (rc) return rc;
  qed3_solve_report r{};
  r.status = int(sc[4]);
  r.iters = int(sc[2]);
  r.reliable_updates = int(sc[3]);
  r.true_rel_res = sc[1] > 0 ? std::sqrt(sc[0] / sc[1]) : 0.0;
  float ms = 0.f;
  QED3_CUDA_TRY(cudaEventElapsedTime(&ms, w.e0, w.e1));
  r.ms = ms;
  d->last = r;
  if (rep) *rep = r;
  if (r.status == QED3_ERR_TIMEOUT) return fail(QED3_ERR_TIMEOUT, "grid barrier timed out inside the CG kernel");
  return QED3_OK;
}

}  // namespace qed3
