"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle is the FP64 CPU restatement of the reference's fermion hot path
(see oracle.cpp for the reference file:line of every routine).  Only tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs
may import this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (a second or two)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "oracle.cpp")
    ):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        L.orc_geom_create.restype = vp
        L.orc_geom_create.argtypes = [ctypes.c_int]
        L.orc_geom_destroy.argtypes = [vp]
        L.orc_geom_sizes.argtypes = [vp] + [c_int_p] * 5
        L.orc_geom_get.argtypes = [vp] + [ctypes.c_void_p] * 13
        L.orc_check_spin_structure.restype = ctypes.c_double
        L.orc_check_spin_structure.argtypes = [vp]
        L.orc_check_deficits.restype = ctypes.c_int
        L.orc_check_deficits.argtypes = [vp, c_double_p]
        L.orc_dirac_create.restype = vp
        L.orc_dirac_create.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.orc_dirac_destroy.argtypes = [vp]
        L.orc_dirac_update.argtypes = [vp, vp, c_double_p]
        L.orc_dirac_apply.argtypes = [vp, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_dirac_nnz.restype = ctypes.c_int
        L.orc_dirac_nnz.argtypes = [vp]
        L.orc_dirac_get_csr.argtypes = [vp, c_int_p, c_int_p, ctypes.c_void_p]
        L.orc_dirac_get_csr_dagger.argtypes = [vp, c_int_p, c_int_p, ctypes.c_void_p]
        L.orc_dirac_get_kappa.argtypes = [vp, c_double_p]
        L.orc_bicgstab.restype = ctypes.c_int
        L.orc_bicgstab.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_double, c_int_p]
        L.orc_cg.restype = ctypes.c_int
        L.orc_cg.argtypes = [vp, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                             ctypes.c_int, c_double_p]
        L.orc_zolotarev.restype = ctypes.c_int
        L.orc_zolotarev.argtypes = [ctypes.c_double, ctypes.c_int] + [c_double_p] * 4
        L.orc_plaquettes.argtypes = [vp, c_double_p, c_double_p]
        L.orc_gauge_action.restype = ctypes.c_double
        L.orc_gauge_action.argtypes = [vp, c_double_p, ctypes.c_double, ctypes.c_int]
        L.orc_gauge_force.argtypes = [vp, c_double_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, c_double_p]
        L.orc_rng_create.restype = vp
        L.orc_rng_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_rng_destroy.argtypes = [vp]
        L.orc_rng_gaussian_links.argtypes = [vp, ctypes.c_double, c_double_p]
        L.orc_rng_gaussian_spinor.argtypes = [vp, ctypes.c_void_p]
        L.orc_rng_gaussian_sites.argtypes = [vp, ctypes.c_double, c_double_p]
        L.orc_rng_z2_spinor.argtypes = [vp, ctypes.c_void_p]
        L.orc_rng_uniform.restype = ctypes.c_double
        L.orc_rng_uniform.argtypes = [vp]
        L.orc_hmc_pure_gauge.restype = ctypes.c_int
        L.orc_hmc_pure_gauge.argtypes = [vp, vp, c_double_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int, c_double_p]
        L.orc_fermion_force.argtypes = [vp, vp, c_double_p, ctypes.c_void_p, c_double_p]
        L.orc_fermion_force_chi.argtypes = [vp, vp, c_double_p, ctypes.c_void_p, ctypes.c_void_p, c_double_p]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_hmc_fermion.restype = ctypes.c_int
        L.orc_hmc_fermion.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_int, vp, vp]
        L.orc_overlap_force.restype = ctypes.c_int
        L.orc_overlap_force.argtypes = [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, vp, vp,
                                        ctypes.c_double]
        L.orc_overlap_apply.restype = ctypes.c_int
        L.orc_overlap_apply.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]
        L.orc_lambda_bounds.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.c_double, c_double_p, c_double_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _dp(a):
    return a.ctypes.data_as(c_double_p)


@dataclass
class Geometry:
    n: int
    sites: np.ndarray
    nns: np.ndarray
    links: np.ndarray
    simp_links: np.ndarray
    simp_sites: np.ndarray
    face_offsets: np.ndarray
    face_sites: np.ndarray
    ell: np.ndarray
    link_volume: np.ndarray
    vols: np.ndarray
    omega: np.ndarray
    alpha: np.ndarray
    mean_ell: float
    mean_link_volume: float
    mean_vol: float
    handle: int = 0

    @property
    def n_sites(self):
        return self.sites.shape[0]

    @property
    def n_links(self):
        return self.links.shape[0]

    @property
    def n_faces(self):
        return self.vols.shape[0]

    def faces(self):
        return [self.face_sites[self.face_offsets[i]:self.face_offsets[i + 1]] for i in range(self.n_faces)]

    def spin_structure_residual(self) -> float:
        return lib().orc_check_spin_structure(self.handle)

    def deficits(self):
        sums = np.zeros(self.n_faces)
        bad = lib().orc_check_deficits(self.handle, _dp(sums))
        return bad, sums

    def __del__(self):
        if self.handle and _lib is not None:
            _lib.orc_geom_destroy(self.handle)
            self.handle = 0


def geometry(n: int) -> Geometry:
    L = lib()
    h = L.orc_geom_create(n)
    if not h:
        raise RuntimeError(f"oracle geometry failed for n={n}")
    ns, nl, nf, nv, ft = (ctypes.c_int() for _ in range(5))
    L.orc_geom_sizes(h, ctypes.byref(ns), ctypes.byref(nl), ctypes.byref(nf), ctypes.byref(nv), ctypes.byref(ft))
    Ns, Nl, Nv, Ft = ns.value, nl.value, nv.value, ft.value
    sites = np.zeros((Ns, 3))
    nns = np.zeros((Ns, 3), np.int32)
    links = np.zeros((Nl, 2), np.int32)
    simp_links = np.zeros((Nl, 2), np.int32)
    simp_sites = np.zeros((Nv, 3))
    face_off = np.zeros(Nv + 1, np.int32)
    face_sites = np.zeros(Ft, np.int32)
    ell = np.zeros(Nl)
    lv = np.zeros(Nl)
    vols = np.zeros(Nv)
    omega = np.zeros(Nl)
    alpha = np.zeros((Ns, 3))
    means = np.zeros(3)
    L.orc_geom_get(h, *[_p(a) for a in (sites, nns, links, simp_links, simp_sites, face_off, face_sites, ell, lv,
                                         vols, omega, alpha, means)])
    return Geometry(n, sites, nns, links, simp_links, simp_sites, face_off, face_sites, ell, lv, vols, omega, alpha,
                    float(means[0]), float(means[1]), float(means[2]), h)


class Dirac:
    """Reference CSR operator D (and D^dagger) on the dual lattice, Nt=1."""

    def __init__(self, geom: Geometry, r: float = 1.0, M5: float = 0.0):
        self.geom = geom
        self.N = 2 * geom.n_sites
        self.h = lib().orc_dirac_create(geom.handle, r, M5)

    def update(self, A: np.ndarray):
        A = np.ascontiguousarray(A, dtype=np.float64)
        lib().orc_dirac_update(self.h, self.geom.handle, _dp(A))

    def apply(self, v: np.ndarray, op: int = 0) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        out = np.zeros_like(v)
        lib().orc_dirac_apply(self.h, op, _p(out), _p(v))
        return out

    def kappa(self):
        k = np.zeros(self.geom.n_links)
        lib().orc_dirac_get_kappa(self.h, _dp(k))
        return k

    def dense(self) -> np.ndarray:
        nnz = lib().orc_dirac_nnz(self.h)
        rows = np.zeros(self.N + 1, np.int32)
        cols = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        lib().orc_dirac_get_csr(self.h, rows.ctypes.data_as(c_int_p), cols.ctypes.data_as(c_int_p), _p(val))
        M = np.zeros((self.N, self.N), np.complex128)
        for i in range(self.N):
            for jj in range(rows[i], rows[i + 1]):
                M[i, cols[jj]] += val[jj]
        return M

    def csr(self, dagger: bool = False):
        """DWDevice's CSR arrays (rows, cols, complex values) of D, or of D^dagger."""
        nnz = lib().orc_dirac_nnz(self.h)
        rows = np.zeros(self.N + 1, np.int32)
        cols = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        f = lib().orc_dirac_get_csr_dagger if dagger else lib().orc_dirac_get_csr
        f(self.h, rows.ctypes.data_as(c_int_p), cols.ctypes.data_as(c_int_p), _p(val))
        return rows, cols, val

    def cg(self, b: np.ndarray, tol: float = 1e-10, maxiter: int = 100000, shift: float = 0.0):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        mu = ctypes.c_double()
        it = lib().orc_cg(self.h, shift, _p(x), _p(b), tol, maxiter, ctypes.byref(mu))
        return x, it, mu.value

    def bicgstab(self, b: np.ndarray, op: int = 0, tol: float = 1e-10, maxiter: int = 100000, shift: float = 0.0,
                 eps: float = 1e-8):
        """MatPoly::bicgstab restated on (op + shift) x = b; returns (x, iterations, converged)."""
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        st = ctypes.c_int()
        it = lib().orc_bicgstab(self.h, op, shift, _p(x), _p(b), tol, maxiter, eps, ctypes.byref(st))
        return x, it, st.value == 0

    def fermion_force(self, A: np.ndarray, eta: np.ndarray) -> np.ndarray:
        A = np.ascontiguousarray(A, dtype=np.float64)
        eta = np.ascontiguousarray(eta, dtype=np.complex128)
        F = np.zeros(self.geom.n_links)
        lib().orc_fermion_force(self.h, self.geom.handle, _dp(A), _p(eta), _dp(F))
        return F

    def fermion_force_chi(self, A: np.ndarray, chi: np.ndarray, eta: np.ndarray) -> np.ndarray:
        """F_l = -2 Re <chi, dD/dA_l eta> (fermion_force with D eta replaced by chi)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        chi = np.ascontiguousarray(chi, dtype=np.complex128)
        eta = np.ascontiguousarray(eta, dtype=np.complex128)
        F = np.zeros(self.geom.n_links)
        lib().orc_fermion_force_chi(self.h, self.geom.handle, _dp(A), _p(chi), _p(eta), _dp(F))
        return F

    def overlap(self, v: np.ndarray, lmin: float, lmax: float, order: int = 21, op: int = 0,
                tol_inner: float = 1e-12) -> np.ndarray:
        """Overlap::mult (op 0) / adj (1) / DHD (2) restated, CG per pole."""
        v = np.ascontiguousarray(v, dtype=np.complex128)
        out = np.zeros_like(v)
        lib().orc_overlap_apply(self.h, lmin, lmax, order, op, _p(out), _p(v), tol_inner)
        return out

    def overlap_force(self, A: np.ndarray, eta: np.ndarray, lmin: float, lmax: float, order: int = 21,
                      tol_inner: float = 1e-12) -> np.ndarray:
        """Overlap::precalc_grad + grad_deviceAsyncLaunch restated: F_l = -2 d/dA_l Re<eta, D_ov eta>."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        eta = np.ascontiguousarray(eta, dtype=np.complex128)
        F = np.zeros(self.geom.n_links)
        lib().orc_overlap_force(self.h, self.geom.handle, _dp(A), lmin, lmax, order, _p(eta), _dp(F), tol_inner)
        return F

    def lambda_bounds(self, TOL: float = 1e-8, maxiter: int = 500, tol_outer: float = 1e-10):
        """Overlap::compute_lambda_max restated: (lambda_min, lambda_max) of D."""
        a, b = ctypes.c_double(), ctypes.c_double()
        lib().orc_lambda_bounds(self.h, TOL, maxiter, tol_outer, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def __del__(self):
        if getattr(self, "h", 0) and _lib is not None:
            _lib.orc_dirac_destroy(self.h)
            self.h = 0


def zolotarev(k: float, n: int):
    size = n // 2 + 1
    c, cp, A, sc = np.zeros(size), np.zeros(size), np.zeros(size), np.zeros(4)
    lib().orc_zolotarev(k, n, _dp(c), _dp(cp), _dp(A), _dp(sc))
    return dict(c=c, cp=cp, A=A, M=sc[0], lambda_inv=sc[1], E=sc[2], C=sc[3], size=size, k=k, n=n)


def zolotarev_eval(z: dict, x):
    """r(x) = C x (1 + sum_m A_m / (x^2 - k^2/cp_m)), src/both_3d/overlap.h:123-128."""
    x = np.asarray(x, dtype=np.float64)
    res = np.ones_like(x)
    for m in range(1, z["size"]):
        res = res + z["A"][m] / (x * x - z["k"] ** 2 / z["cp"][m])
    return res * z["C"] * x


def plaquettes(geom: Geometry, A):
    A = np.ascontiguousarray(A, dtype=np.float64)
    th = np.zeros(geom.n_faces)
    lib().orc_plaquettes(geom.handle, _dp(A), _dp(th))
    return th


def gauge_action(geom: Geometry, A, beta: float, compact: bool = True) -> float:
    A = np.ascontiguousarray(A, dtype=np.float64)
    return lib().orc_gauge_action(geom.handle, _dp(A), beta, int(compact))


def gauge_force(geom: Geometry, A, beta: float, compact: bool = True, exact: bool = True):
    A = np.ascontiguousarray(A, dtype=np.float64)
    F = np.zeros(geom.n_links)
    lib().orc_gauge_force(geom.handle, _dp(A), beta, int(compact), int(exact), _dp(F))
    return F


class Rng:
    """ParallelRng2 restated: master mt19937_64 seeds per-link then per-site engines."""

    def __init__(self, geom: Geometry, seed: int, n_slices: int = 1):
        """n_slices > 1: ParallelRngExt (src/both_3d/rng.h:89-121), engines
        [Nt][n_links] and [Nt][n_sites] seeded in that order (flat order = the
        layout of one ParallelRng2 with Nt times as many links and sites)."""
        self.geom = geom
        self.nl, self.ns = geom.n_links * n_slices, geom.n_sites * n_slices
        self.h = lib().orc_rng_create(self.nl, self.ns, seed)

    def gaussian_links(self, width=1.0):
        out = np.zeros(self.nl)
        lib().orc_rng_gaussian_links(self.h, width, _dp(out))
        return out

    def gaussian_sites(self, width=1.0):
        out = np.zeros(self.ns)
        lib().orc_rng_gaussian_sites(self.h, width, _dp(out))
        return out

    def gaussian_spinor(self):
        out = np.zeros(2 * self.ns, np.complex128)
        lib().orc_rng_gaussian_spinor(self.h, _p(out))
        return out

    def z2_spinor(self):
        """FermionVector::set_random (src/dual/valence.h:54-60)."""
        out = np.zeros(2 * self.ns, dtype=np.complex128)
        lib().orc_rng_z2_spinor(self.h, _p(out))
        return out

    def uniform(self):
        return lib().orc_rng_uniform(self.h)

    def __del__(self):
        if getattr(self, "h", 0) and _lib is not None:
            _lib.orc_rng_destroy(self.h)
            self.h = 0


def hmc_pure_gauge(geom: Geometry, rng: Rng, A: np.ndarray, beta: float, compact=True, exact=True, tmax=1.0,
                   nsteps=40, no_reject=False):
    """One HMCPureGauge trajectory in place on A; returns (accepted, dH)."""
    assert A.dtype == np.float64 and A.flags.c_contiguous
    dH = ctypes.c_double()
    acc = lib().orc_hmc_pure_gauge(geom.handle, rng.h, _dp(A), beta, int(compact), int(exact), tmax, nsteps,
                                   int(no_reject), ctypes.byref(dH))
    return bool(acc), dH.value


def thermalized_links(geom: Geometry, beta: float, seed: int, ntraj: int, init: str = "gaussian",
                      compact: bool = True, exact: bool = True, nsteps: int = 40):
    """Seeded pure-gauge configuration (src/both/gauge.cu:157-200 recipe)."""
    rng = Rng(geom, seed)
    if init == "gaussian":
        A = rng.gaussian_links(0.2)
    elif init == "uniform":
        r = np.random.default_rng(seed)
        A = r.uniform(-np.pi, np.pi, geom.n_links)
    else:
        A = np.zeros(geom.n_links)
    A = np.ascontiguousarray(A)
    acc = 0
    for _ in range(ntraj):
        a, _ = hmc_pure_gauge(geom, rng, A, beta, compact, exact, 1.0, nsteps)
        acc += a
    return A, acc


def num_threads() -> int:
    return lib().orc_num_threads()


def hmc_fermion(geom: Geometry, dirac: "Dirac", rng: "Rng", A: np.ndarray, beta: float, compact: bool = True,
                exact: bool = True, tmax: float = 1.0, nsteps: int = 10, nsteps_inner: int = 10, tol: float = 1e-12,
                no_reject: bool = False, npf: int = 1, integrator: int = 0):
    """HMC::run (npf = 1) or HMC2::run (npf pseudofermions) with ExplicitLeapfrogML
    (integrator 0) or ExplicitLeapfrog (1) restated; A updated in place.
    Returns (accepted, dH, cg_iterations)."""
    dH = ctypes.c_double()
    its = ctypes.c_int()
    acc = lib().orc_hmc_fermion(geom.handle, dirac.h, rng.h, _dp(A), beta, int(compact), 1 if exact else 0, tmax,
                                nsteps, nsteps_inner, npf, integrator, tol, int(no_reject), ctypes.byref(dH),
                                ctypes.byref(its))
    return bool(acc), dH.value, its.value


def hmc_overlap(geom: Geometry, dirac: "Dirac", rng: "Rng", A: np.ndarray, beta: float, compact: bool = True,
                exact: bool = True, tmax: float = 1.0, nsteps: int = 10, nsteps_inner: int = 10, npf: int = 1,
                lmin: float = 0.0, lmax: float = 0.0, order: int = 21, tol: float = 1e-10, tol_inner: float = 1e-12,
                no_reject: bool = False, integrator: int = 0):
    """HMC2::run with Overlap fermions (src/both_3d/hmc.h:172-200, src/both_3d/hmc.cu:155-160)
    and ExplicitLeapfrogML (src/both_3d/integrator.h:117-168), composed from the
    oracle's overlap pieces; A updated in place.  lmin = lmax = 0: every operator
    update recomputes the bounds (Overlap::update, src/both_3d/overlap.h:207-216).
    eta = (D_ov^dag D_ov)^{-1} phi by MatPoly::solve's CG (src/dual/matpoly.h:204-267)
    on Overlap::DHD.  Returns (accepted, dH, outer CG iterations)."""
    fixed = lmin > 0 or lmax > 0
    bounds = [lmin, lmax]
    pi = rng.gaussian_links(1.0)
    xis = [rng.gaussian_spinor() for _ in range(npf)]
    A0 = A.copy()

    def update():
        dirac.update(A)
        if not fixed:
            bounds[0], bounds[1] = dirac.lambda_bounds(tol_outer=tol_inner)

    def ov(v, op):
        return dirac.overlap(v, bounds[0], bounds[1], order, op, tol_inner=tol_inner)

    its = [0]

    def solve(b):
        x = np.zeros_like(b)
        r = b.copy()
        p = r.copy()
        bb = np.vdot(b, b).real
        rr = bb
        while True:
            q = ov(p, 2)
            al = rr / np.vdot(p, q).real
            x += al * p
            r -= al * q
            rn = np.vdot(r, r).real
            its[0] += 1
            if rn < tol * tol * bb:
                return x
            p = r + (rn / rr) * p
            rr = rn

    update()
    phis = [ov(xi, 1) for xi in xis]
    etas = [solve(ph) for ph in phis]

    def H():
        return (0.5 * float(np.dot(pi, pi)) + gauge_action(geom, A, beta, compact)
                + sum(np.vdot(ph, et).real for ph, et in zip(phis, etas)))

    h0 = H()
    tau = tmax / nsteps
    tau_in = tau / nsteps_inner

    def full_force():  # dSg + dSf, the single-level ExplicitLeapfrog's kick
        Fs = gauge_force(geom, A, beta, compact, exact)
        for k in range(npf):
            Fs = Fs + dirac.overlap_force(A, etas[k], bounds[0], bounds[1], order, tol_inner)
        return Fs

    if integrator == 1:
        for n in range(nsteps):
            pi += -0.5 * tau * full_force()
            A += tau * pi
            update()
            for k in range(npf):
                etas[k] = solve(phis[k])
            pi += -0.5 * tau * full_force()
        nsteps_ml = 0
    else:
        nsteps_ml = nsteps
    for k in range(npf if integrator != 1 else 0):
        pi -= 0.5 * tau * dirac.overlap_force(A, etas[k], bounds[0], bounds[1], order, tol_inner)
    for n in range(nsteps_ml):
        pi -= 0.5 * tau_in * gauge_force(geom, A, beta, compact, exact)
        for m in range(nsteps_inner):
            A += tau_in * pi
            pi -= (1.0 if m != nsteps_inner - 1 else 0.5) * tau_in * gauge_force(geom, A, beta, compact, exact)
        update()
        for k in range(npf):
            etas[k] = solve(phis[k])
            pi -= (1.0 if n != nsteps - 1 else 0.5) * tau * dirac.overlap_force(A, etas[k], bounds[0], bounds[1],
                                                                                 order, tol_inner)
    dH = H() - h0
    r = min(1.0, np.exp(-dH))
    if rng.uniform() < r or no_reject:
        return True, dH, its[0]
    A[:] = A0
    update()
    return False, dH, its[0]


def triangle_areas(geom: Geometry) -> np.ndarray:
    """S2Simp::vols (src/both_3d/s2n_simp.h:234-253): L'Huilier area of the
    simplicial triangle of each dual site (the three dual faces containing it)."""
    tri = [[] for _ in range(geom.n_sites)]
    for f in range(geom.n_faces):
        for x in geom.face_sites[geom.face_offsets[f]:geom.face_offsets[f + 1]]:
            tri[x].append(f)
    out = np.zeros(geom.n_sites)
    for t, (i0, i1, i2) in enumerate(tri):
        x0, x1, x2 = geom.simp_sites[i0], geom.simp_sites[i1], geom.simp_sites[i2]
        a, b, c = np.arccos(x0 @ x1), np.arccos(x1 @ x2), np.arccos(x2 @ x0)
        s = 0.5 * (a + b + c)
        out[t] = 4.0 * np.arctan(np.sqrt(np.tan(0.5 * s) * np.tan(0.5 * (s - a)) * np.tan(0.5 * (s - b))
                                         * np.tan(0.5 * (s - c))))
    return out


def dirac_ext_apply(geom: Geometry, r: float, M5: float, Nt: int, at: float, A: np.ndarray, v: np.ndarray,
                    op: int = 0) -> np.ndarray:
    """DiracExt::coo_format (src/both_3d/dirac_ext.h:121-213) restated as an apply:
    op 0 = D, 1 = D^dag, 2 = D^dag D on v[Nt][Ns][2]; A = spatial [Nt][Nl] then
    temporal [Nt][Ns].  The spatial part of each slice is the dual-lattice
    operator of that slice's links (Dirac.apply); kappa_t = area / mean_ell / at."""
    if op == 2:
        return dirac_ext_apply(geom, r, M5, Nt, at, A, dirac_ext_apply(geom, r, M5, Nt, at, A, v, 0), 1)
    Ns, Nl = geom.n_sites, geom.n_links
    v = np.asarray(v, np.complex128).reshape(Nt, Ns, 2)
    As = np.asarray(A[:Nt * Nl]).reshape(Nt, Nl)
    At = np.asarray(A[Nt * Nl:Nt * (Nl + Ns)]).reshape(Nt, Ns)
    kt = triangle_areas(geom) / geom.mean_ell / at if Nt != 1 else np.zeros(Ns)
    D = Dirac(geom, r, M5)
    out = np.zeros_like(v)
    for s in range(Nt):
        D.update(As[s])
        out[s] = D.apply(v[s].reshape(-1), op).reshape(Ns, 2) + (r * kt)[:, None] * v[s]
    if Nt > 1:
        sig3 = np.array([1.0, -1.0])
        for s in range(Nt):  # the COO entries of column slice s
            sP = -1.0 if s == Nt - 1 else 1.0
            sM = -1.0 if s == 0 else 1.0
            tmpP = 0.5 * sP * kt[:, None] * (-r - sig3)[None, :] * np.exp(-1j * At[s])[:, None]
            tmpM = 0.5 * sM * kt[:, None] * (-r + sig3)[None, :] * np.exp(1j * At[(s - 1) % Nt])[:, None]
            up, dn = (s + 1) % Nt, (s - 1) % Nt
            if op == 0:  # D[(x,s+1),(x,s)] = tmpP(s), D[(x,s-1),(x,s)] = tmpM(s)
                out[up] += tmpP * v[s]
                out[dn] += tmpM * v[s]
            else:  # D^dag[(x,s),(x,s+1)] = conj(tmpP(s)), D^dag[(x,s),(x,s-1)] = conj(tmpM(s))
                out[s] += np.conj(tmpP) * v[up] + np.conj(tmpM) * v[dn]
    return out.reshape(-1)


def ext_gauge(geom: Geometry, Nt: int, at: float, gsq: float, A: np.ndarray):
    """U1WilsonExt restated (src/both_3d/action_ext.h:31-161) with GaugeExt's
    plaquettes (src/both_3d/gauge_ext.h:124-143), loop for loop in the
    reference's order.  Returns (theta_s [Nt][Nf], theta_t [Nt][Nl], S, F) with F
    in A's layout (spatial [Nt][Nl], then temporal [Nt][Ns])."""
    Ns, Nl, Nf = geom.n_sites, geom.n_links, geom.n_faces
    sp = np.asarray(A[:Nt * Nl]).reshape(Nt, Nl)
    tp = np.asarray(A[Nt * Nl:Nt * (Nl + Ns)]).reshape(Nt, Ns)
    il = {(int(i), int(j)): (l, 1) for l, (i, j) in enumerate(geom.links)}
    il.update({(int(j), int(i)): (l, -1) for l, (i, j) in enumerate(geom.links)})
    faces = geom.faces()
    bs = np.array([at / geom.vols[f] / gsq for f in range(Nf)]) if abs(gsq) > 1e-15 else np.zeros(Nf)
    bt = np.array([2.0 / at * geom.link_volume[l] / geom.ell[l] ** 2 / gsq for l in range(Nl)]) \
        if abs(gsq) > 1e-15 else np.zeros(Nl)

    def th_s(s, f):
        t = 0.0
        face = faces[f]
        for k in range(len(face)):
            l, sg = il[(int(face[k]), int(face[(k + 1) % len(face)]))]
            t += sg * sp[s % Nt][l]
        return t

    def th_t(s, l):
        x, y = int(geom.links[l][0]), int(geom.links[l][1])
        t = 0.0
        t += sp[s % Nt][l]
        t += tp[s % Nt][y]
        t -= sp[(s + 1) % Nt][l]
        t -= tp[s % Nt][x]
        return t

    ths = np.array([[th_s(s, f) for f in range(Nf)] for s in range(Nt)])
    tht = np.array([[th_t(s, l) for l in range(Nl)] for s in range(Nt)])
    tmp = [0.0] * Nt
    for s in range(Nt):
        for f in range(Nf):
            tmp[s] += 0.5 * bs[f] * ths[s][f] ** 2
    for s in range(Nt):
        for l in range(Nl):
            tmp[s] += 0.5 * bt[l] * tht[s][l] ** 2
    S = 0.0
    for s in range(Nt):
        S += tmp[s]
    Fs = np.zeros((Nt, Nl))
    Ft = np.zeros((Nt, Ns))
    for s in range(Nt):
        for f in range(Nf):
            grad = bs[f] * ths[s][f]
            face = faces[f]
            for k in range(len(face)):
                l, sg = il[(int(face[k]), int(face[(k + 1) % len(face)]))]
                Fs[s][l] += grad * sg
    for s in range(Nt):
        for l in range(Nl):
            x, y = int(geom.links[l][0]), int(geom.links[l][1])
            grad = bt[l] * tht[s][l]
            grad2 = bt[l] * tht[(s - 1) % Nt][l]
            Fs[s][l] += grad
            Ft[s][y] += grad
            Fs[s][l] -= grad2
            Ft[s][x] -= grad
    return ths, tht, S, np.concatenate([Fs.ravel(), Ft.ravel()])


def ext_polyakov(geom: Geometry, Nt: int, A: np.ndarray) -> np.ndarray:
    """get_polyakov (src/both_3d/obs.h:4-10) at every dual site."""
    Ns, Nl = geom.n_sites, geom.n_links
    tp = np.asarray(A[Nt * Nl:Nt * (Nl + Ns)]).reshape(Nt, Ns)
    out = np.zeros(Ns, np.complex128)
    for x in range(Ns):
        a = 0.0
        for s in range(Nt):
            a += tp[s][x]
        out[x] = np.exp(1j * a)
    return out


def _ext_temporal(geom: Geometry, r: float, Nt: int, at: float, At: np.ndarray):
    """The temporal COO entries of DiracExt (src/both_3d/dirac_ext.h:121-213):
    column slice s couples to row slice s+1 by tmpP[s] and to s-1 by tmpM[s]
    (spin-diagonal, [Nt][Ns][2]), antiperiodic across the boundary."""
    kt = triangle_areas(geom) / geom.mean_ell / at
    sig3 = np.array([1.0, -1.0])
    tmpP = np.empty((Nt, geom.n_sites, 2), np.complex128)
    tmpM = np.empty_like(tmpP)
    for s in range(Nt):
        sP = -1.0 if s == Nt - 1 else 1.0
        sM = -1.0 if s == 0 else 1.0
        tmpP[s] = 0.5 * sP * kt[:, None] * (-r - sig3)[None, :] * np.exp(-1j * At[s])[:, None]
        tmpM[s] = 0.5 * sM * kt[:, None] * (-r + sig3)[None, :] * np.exp(1j * At[(s - 1) % Nt])[:, None]
    return kt, tmpP, tmpM


def dirac_ext_matrix(geom: Geometry, r: float, M5: float, Nt: int, at: float, A: np.ndarray) -> np.ndarray:
    """The dense DiracExt matrix, the same entries as dirac_ext_apply (op 0)."""
    Ns, Nl = geom.n_sites, geom.n_links
    As = np.asarray(A[:Nt * Nl]).reshape(Nt, Nl)
    At = np.asarray(A[Nt * Nl:Nt * (Nl + Ns)]).reshape(Nt, Ns)
    n2 = 2 * Ns
    M = np.zeros((Nt * n2, Nt * n2), np.complex128)
    D = Dirac(geom, r, M5)
    kt, tmpP, tmpM = _ext_temporal(geom, r, Nt, at, At) if Nt > 1 else (np.zeros(Ns), None, None)
    for s in range(Nt):
        D.update(As[s])
        M[s * n2:(s + 1) * n2, s * n2:(s + 1) * n2] = D.dense() + np.diag(np.repeat(r * kt, 2))
    if Nt > 1:
        idx = np.arange(n2)
        for s in range(Nt):
            up, dn = (s + 1) % Nt, (s - 1) % Nt
            M[up * n2 + idx, s * n2 + idx] += tmpP[s].reshape(-1)
            M[dn * n2 + idx, s * n2 + idx] += tmpM[s].reshape(-1)
    return M


def ext_fermion_force(geom: Geometry, r: float, M5: float, Nt: int, at: float, A: np.ndarray, eta: np.ndarray,
                      M: np.ndarray | None = None, chi: np.ndarray | None = None) -> np.ndarray:
    """F = -2 Re <D eta, dD/dA eta> of DiracExt in A's layout: spatial links of
    slice s by the dual-lattice force with chi = (D eta)_s; temporal link (s, x)
    from its two entries, tmpP[s] (row s+1, column s, phase e^{-i A_t}) and
    tmpM[s+1] (row s, column s+1, phase e^{+i A_t})."""
    Ns, Nl = geom.n_sites, geom.n_links
    n2 = 2 * Ns
    eta = np.asarray(eta, np.complex128)
    if chi is None:  # -2 Re <chi, dD/dA eta> with chi = D eta; any chi gives the bilinear form
        M = dirac_ext_matrix(geom, r, M5, Nt, at, A) if M is None else M
        chi = M @ eta
    chi = np.asarray(chi, np.complex128)
    As = np.asarray(A[:Nt * Nl]).reshape(Nt, Nl)
    At = np.asarray(A[Nt * Nl:Nt * (Nl + Ns)]).reshape(Nt, Ns)
    D = Dirac(geom, r, M5)
    Fs = np.zeros((Nt, Nl))
    for s in range(Nt):
        D.update(As[s])
        Fs[s] = D.fermion_force_chi(As[s], chi[s * n2:(s + 1) * n2], eta[s * n2:(s + 1) * n2])
    Ft = np.zeros((Nt, Ns))
    if Nt > 1:
        _, tmpP, tmpM = _ext_temporal(geom, r, Nt, at, At)
        e3, c3 = eta.reshape(Nt, Ns, 2), chi.reshape(Nt, Ns, 2)
        for s in range(Nt):
            up = (s + 1) % Nt
            t = (np.conj(c3[up]) * (-1j) * tmpP[s] * e3[s]).sum(1) + (np.conj(c3[s]) * 1j * tmpM[up] * e3[up]).sum(1)
            Ft[s] = -2.0 * t.real
    return np.concatenate([Fs.ravel(), Ft.ravel()])


def hmc_ext(geom: Geometry, rng: Rng, A: np.ndarray, r: float, M5: float, Nt: int, at: float, gsq: float,
            tmax: float = 1.0, nsteps: int = 4, nsteps_inner: int = 4, npf: int = 1, integrator: int = 0,
            tol: float = 1e-12, no_reject: bool = False):
    """HMC2::run (src/both_3d/hmc.h:172-200) on S^2 x S^1 with U1WilsonExt and
    npf DiracExt pseudofermions; ExplicitLeapfrogML (src/both_3d/integrator.h:117-168)
    or, integrator = 1, ExplicitLeapfrog.  rng = Rng(geom, seed, Nt): momenta by
    GaugeExt::gaussian (src/both_3d/gauge_ext.h:146-149), sources by
    ParallelRngExt::fill_gaussian.  eta = (D^dag D)^{-1} phi by CG on the dense
    operator.  A updated in place; returns (accepted, dH, CG iterations)."""
    Ns, Nl = geom.n_sites, geom.n_links
    pi = np.concatenate([rng.gaussian_links(1.0), rng.gaussian_sites(1.0)])
    xis = [rng.gaussian_spinor() for _ in range(npf)]
    A0 = A.copy()
    st = {"M": dirac_ext_matrix(geom, r, M5, Nt, at, A)}
    its = [0]

    def solve(b):
        M = st["M"]
        x = np.zeros_like(b)
        rr_ = b.copy()
        p = rr_.copy()
        bb = np.vdot(b, b).real
        rr = bb
        while rr > tol * tol * bb:
            q = M.conj().T @ (M @ p)
            al = rr / np.vdot(p, q).real
            x += al * p
            rr_ -= al * q
            rn = np.vdot(rr_, rr_).real
            its[0] += 1
            p = rr_ + (rn / rr) * p
            rr = rn
        return x

    phis = [st["M"].conj().T @ xi for xi in xis]
    etas = [solve(ph) for ph in phis]

    def H():
        return (0.5 * float(np.dot(pi, pi)) + ext_gauge(geom, Nt, at, gsq, A)[2]
                + sum(np.vdot(ph, et).real for ph, et in zip(phis, etas)))

    def update():
        st["M"] = dirac_ext_matrix(geom, r, M5, Nt, at, A)
        for k in range(npf):
            etas[k] = solve(phis[k])

    gforce = lambda: ext_gauge(geom, Nt, at, gsq, A)[3]
    fforce = lambda k: ext_fermion_force(geom, r, M5, Nt, at, A, etas[k], st["M"])
    h0 = H()
    tau = tmax / nsteps
    tau_in = tau / nsteps_inner
    if integrator == 1:
        for n in range(nsteps):
            pi -= 0.5 * tau * (gforce() + sum(fforce(k) for k in range(npf)))
            A += tau * pi
            update()
            pi -= 0.5 * tau * (gforce() + sum(fforce(k) for k in range(npf)))
    else:
        for k in range(npf):
            pi -= 0.5 * tau * fforce(k)
        for n in range(nsteps):
            pi -= 0.5 * tau_in * gforce()
            for m in range(nsteps_inner):
                A += tau_in * pi
                pi -= (1.0 if m != nsteps_inner - 1 else 0.5) * tau_in * gforce()
            update()
            for k in range(npf):
                pi -= (1.0 if n != nsteps - 1 else 0.5) * tau * fforce(k)
    h1 = H()
    dH = h1 - h0
    a = rng.uniform()
    if a < min(1.0, np.exp(-dH)) or no_reject:
        return True, dH, its[0]
    A[:] = A0
    return False, dH, its[0]


def dirac1f_tables(geom: Geometry):
    """The u, v tables of integrator/test_sorting.cc:499-594 (us_*, vs_*):
    per site x, hop vectors ell_k = acos(x . y_k) (cos alpha_k, sin alpha_k);
    v from [d13 d23] (v1_c, v2_c) = (a/sqrt3) e_c, v3 = -v1 - v2,
    a = sqrt(4/sqrt3 vbar), vbar the mean triangle area; u = (1, p, q) with
    [ell2 ell3](p, q) = -ell1, then u *= 3/mean(u).  Returns (u [Ns,3], v [Ns,3,2],
    vol [Ns], vbar), solving each small system with numpy."""
    vol = triangle_areas(geom)
    vbar = float(np.mean(vol))
    alat = np.sqrt(4.0 / np.sqrt(3.0) * vbar)
    Ns = geom.n_sites
    u = np.zeros((Ns, 3))
    v = np.zeros((Ns, 3, 2))
    for x in range(Ns):
        el = []
        for k in range(3):
            y = int(geom.nns[x][k])
            c = float(np.dot(geom.sites[x], geom.sites[y]))
            ln = np.pi if c < -1 else (0.0 if c > 1 else np.arccos(c))
            al = geom.alpha[x][k]
            el.append(ln * np.array([np.cos(al), np.sin(al)]))
        d13, d23 = el[0] - el[2], el[1] - el[2]
        mat = np.array([[d13[0], d23[0], 0, 0], [d13[1], d23[1], 0, 0], [0, 0, d13[0], d23[0]],
                        [0, 0, d13[1], d23[1]]])
        vv = np.linalg.solve(mat, np.array([1.0, 0.0, 0.0, 1.0]) * alat / np.sqrt(3.0))
        v[x, 0] = (vv[0], vv[2])
        v[x, 1] = (vv[1], vv[3])
        v[x, 2] = -v[x, 0] - v[x, 1]
        pq = np.linalg.solve(np.array([[el[1][0], el[2][0]], [el[1][1], el[2][1]]]), -el[0])
        uu = np.array([1.0, pq[0], pq[1]])
        u[x] = uu * (3.0 / uu.mean())
    return u, v, vol, vbar


def dirac1f_matrix(geom: Geometry, r: float, m: float, M5: float, A: np.ndarray) -> np.ndarray:
    """Dirac1fonS2::matrix_form(U) (src/dual/dirac.h:170-183) as a dense matrix:
    block (x, y_k) -= (vol_x/vbar)(r u_k - gamma_k) e^{iU(x,y)} Omega(x,y),
    block (x, x) += (vol_x/vbar)(r u_k + m/3) + M5/3 for each k."""
    u, v, vol, vbar = dirac1f_tables(geom)
    Ns = geom.n_sites
    s1 = np.array([[0, 1], [1, 0]], complex)
    s2 = np.array([[0, -1j], [1j, 0]], complex)
    sgn = {}
    for l, (i, j) in enumerate(geom.links):
        sgn[(int(i), int(j))] = (l, 1.0)
        sgn[(int(j), int(i))] = (l, -1.0)
    M = np.zeros((2 * Ns, 2 * Ns), complex)
    for x in range(Ns):
        for k in range(3):
            y = int(geom.nns[x][k])
            l, sg = sgn[(x, y)]
            om = sg * geom.omega[l]
            Om = np.diag([np.exp(-0.5j * om), np.exp(0.5j * om)])
            gam = v[x, k, 0] * s1 + v[x, k, 1] * s2
            w = vol[x] / vbar
            M[2 * x:2 * x + 2, 2 * y:2 * y + 2] -= w * (r * u[x, k] * np.eye(2) - gam) * np.exp(1j * sg * A[l]) @ Om
            M[2 * x:2 * x + 2, 2 * x:2 * x + 2] += (w * (r * u[x, k] + m / 3.0) + M5 / 3.0) * np.eye(2)
    return M


def overlap_ext_matrix(geom: Geometry, r: float, M5: float, Nt: int, at: float, A: np.ndarray, lmin: float,
                       lmax: float, order: int) -> np.ndarray:
    """Overlap<DiracExt>::mult (src/both_3d/overlap.h:309-332) as a dense matrix:
    D_ov = 1 + C X (1 + sum_m A_m (X^dag X - k^2/cp_m)^{-1}), X = D / lambda_max,
    with the Zolotarev coefficients of `zolotarev` (k = lambda_min / lambda_max)."""
    M = dirac_ext_matrix(geom, r, M5, Nt, at, A)
    z = zolotarev(lmin / lmax, order)
    X = M / lmax
    H = X.conj().T @ X
    I = np.eye(M.shape[0])
    acc = I.copy()
    for m in range(1, z["size"]):
        acc = acc + z["A"][m] * np.linalg.inv(H - z["k"] ** 2 / z["cp"][m] * I)
    return I + z["C"] * X @ acc


def overlap_ext_force(geom: Geometry, r: float, M5: float, Nt: int, at: float, A: np.ndarray, eta: np.ndarray,
                      lmin: float, lmax: float, order: int) -> np.ndarray:
    """-2 d/dA Re<eta, D_ov eta> of Overlap<DiracExt> (Overlap::precalc_grad +
    grad_deviceAsyncLaunch, src/both_3d/overlap.h:393-470) by the chain rule on
    dense matrices: with X = D/lmax, H = X^dag X, z_m = (H + s_m)^{-1} eta,
    y_m = (H + s_m)^{-1} X^dag eta, w = eta + sum_m A_m z_m,
      Re<eta, dD_ov eta> = C/lmax Re<eta, dD w>
                           - C/lmax^2 sum_m A_m (Re<D z_m, dD y_m> + Re<D y_m, dD z_m>),
    each Re<a, dD b> from the bilinear form of ext_fermion_force."""
    M = dirac_ext_matrix(geom, r, M5, Nt, at, A)
    z = zolotarev(lmin / lmax, order)
    X = M / lmax
    H = X.conj().T @ X
    I = np.eye(M.shape[0])
    eta = np.asarray(eta, np.complex128)
    form = lambda a, b: -0.5 * ext_fermion_force(geom, r, M5, Nt, at, A, b, chi=a)  # Re<a, dD b>
    w = eta.copy()
    acc = 0.0
    for m in range(1, z["size"]):
        Hs = H - z["k"] ** 2 / z["cp"][m] * I
        zm = np.linalg.solve(Hs, eta)
        ym = np.linalg.solve(Hs, X.conj().T @ eta)
        w = w + z["A"][m] * zm
        acc = acc + z["A"][m] * (form(M @ zm, ym) + form(M @ ym, zm))
    re = z["C"] / lmax * form(eta, w) - z["C"] / lmax ** 2 * acc
    return -2.0 * re


def hmc_ext_overlap(geom: Geometry, rng: Rng, A: np.ndarray, r: float, M5: float, Nt: int, at: float, gsq: float,
                    lmin: float, lmax: float, order: int, tmax: float = 1.0, nsteps: int = 4, nsteps_inner: int = 4,
                    npf: int = 1, integrator: int = 0, no_reject: bool = False):
    """HMC2::run with Overlap<DiracExt> pseudofermions (the IS_OVERLAP build of
    src/both_3d/hmc.cu) at fixed bounds: hmc_ext with phi = D_ov^dag xi,
    eta = (D_ov^dag D_ov)^{-1} phi solved densely (D_ov^dag D_ov taken as
    D_ov + D_ov^dag, Overlap::DHD), and overlap_ext_force.  A updated in place;
    returns (accepted, dH)."""
    pi = np.concatenate([rng.gaussian_links(1.0), rng.gaussian_sites(1.0)])
    xis = [rng.gaussian_spinor() for _ in range(npf)]
    A0 = A.copy()
    st = {}

    def update():
        Dv = overlap_ext_matrix(geom, r, M5, Nt, at, A, lmin, lmax, order)
        st["D"] = Dv
        st["H"] = Dv + Dv.conj().T

    update()
    phis = [st["D"].conj().T @ xi for xi in xis]
    etas = [np.linalg.solve(st["H"], ph) for ph in phis]

    def H():
        return (0.5 * float(np.dot(pi, pi)) + ext_gauge(geom, Nt, at, gsq, A)[2]
                + sum(np.vdot(ph, et).real for ph, et in zip(phis, etas)))

    def resolve():
        update()
        for k in range(npf):
            etas[k] = np.linalg.solve(st["H"], phis[k])

    gforce = lambda: ext_gauge(geom, Nt, at, gsq, A)[3]
    fforce = lambda k: overlap_ext_force(geom, r, M5, Nt, at, A, etas[k], lmin, lmax, order)
    h0 = H()
    tau = tmax / nsteps
    tau_in = tau / nsteps_inner
    if integrator == 1:
        for n in range(nsteps):
            pi -= 0.5 * tau * (gforce() + sum(fforce(k) for k in range(npf)))
            A += tau * pi
            resolve()
            pi -= 0.5 * tau * (gforce() + sum(fforce(k) for k in range(npf)))
    else:
        for k in range(npf):
            pi -= 0.5 * tau * fforce(k)
        for n in range(nsteps):
            pi -= 0.5 * tau_in * gforce()
            for m in range(nsteps_inner):
                A += tau_in * pi
                pi -= (1.0 if m != nsteps_inner - 1 else 0.5) * tau_in * gforce()
            resolve()
            for k in range(npf):
                pi -= (1.0 if n != nsteps - 1 else 0.5) * tau * fforce(k)
    dH = H() - h0
    a = rng.uniform()
    if a < min(1.0, np.exp(-dH)) or no_reject:
        return True, dH
    A[:] = A0
    return False, dH
