"""qed3-gb300: GB300-native fermion hot path of qed3 behind a C ABI.

The compute path is the in-tree CUDA library ``libqed3.so`` (sm_103a); this
module only binds its C entry points (``include/qed3.h``) with ctypes and
mirrors the reference's object names:

* :class:`S2Trivalent`   -- the dual lattice (src/both_3d/s2n_dual.h:15)
* :class:`DiracS2Dual`   -- Wilson-Dirac operator + its device form
  (src/both_3d/dirac_dual.h:63, src/both_3d/sparse_dirac.h:5)
* :meth:`DiracS2Dual.solve` -- CG on D^dagger D (MatPoly::solve,
  src/dual/matpoly.h:204)

Device vectors are torch CUDA tensors (complex128, reference site order,
index 2*x+s) passed by pointer; torch is only used for device memory and
streams.  There is no CPU fallback: if the library or a GPU is missing,
the calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqed3.so")

OK, ERR_ARG, ERR_CUDA, ERR_NOCONV, ERR_TIMEOUT, ERR_STATE, ERR_NOMEM = range(7)
OP_D, OP_DDAG, OP_DDAGD, OP_DDDAG = range(4)
PREC_F64, PREC_F32, PREC_BF16 = range(3)
INTEGRATOR_LEAPFROG_ML, INTEGRATOR_LEAPFROG = 0, 1
SOLVE_STREAMING = 2
SOLVE_BCAST_B = 4
SOLVE_FLEXIBLE = 8
SOLVE_PIPELINED = 16
OVSOLVE_CHIRAL = 1
POLES_MULTISHIFT, POLES_BATCHED = 0, 1
BATCH_STATIC, BATCH_DYNAMIC = 1, 2
PREC_NAMES = {"f64": PREC_F64, "f32": PREC_F32, "bf16": PREC_BF16}
BYTES_PER_SITE = {PREC_F64: 32, PREC_F32: 16, PREC_BF16: 8}

_lib = None
vp = ctypes.c_void_p
c_int_p = ctypes.POINTER(ctypes.c_int)
c_double_p = ctypes.POINTER(ctypes.c_double)


class SolveParams(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("maxiter", ctypes.c_int), ("precision", ctypes.c_int),
                ("delta", ctypes.c_double), ("shift", ctypes.c_double), ("flags", ctypes.c_int)]


class SolveReport(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iters", ctypes.c_int), ("reliable_updates", ctypes.c_int),
                ("true_rel_res", ctypes.c_double), ("ms", ctypes.c_double)]


class Qed3Error(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"qed3 status {status}: {msg}")
        self.status = status


# (name, restype, argtypes) of every entry point of include/qed3.h
SIGNATURES = [
    ("qed3_last_error_string", ctypes.c_char_p, []),
    ("qed3_version", ctypes.c_int, []),
    ("qed3_selftest_wait_timeout", ctypes.c_int, [ctypes.c_longlong, c_int_p, c_int_p]),
    ("qed3_rng_uniform", ctypes.c_int, [vp, c_double_p]),
    ("qed3_rng_save", ctypes.c_int, [vp, ctypes.c_char_p]),
    ("qed3_rng_load", ctypes.c_int, [vp, ctypes.c_char_p]),
    ("qed3_links_save", ctypes.c_int, [vp, vp, ctypes.c_char_p]),
    ("qed3_links_load", ctypes.c_int, [vp, vp, c_double_p, ctypes.c_char_p]),
    ("qed3_lattice_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(vp)]),
    ("qed3_lattice_destroy", ctypes.c_int, [vp]),
    ("qed3_lattice_sizes", ctypes.c_int, [vp, c_int_p, c_int_p, c_int_p, c_int_p]),
    ("qed3_lattice_tables", ctypes.c_int, [vp] + [vp] * 12),
    ("qed3_lattice_from_mesh", ctypes.c_int, [ctypes.c_int, vp, ctypes.c_int, vp, vp, ctypes.POINTER(vp)]),
    ("qed3_lattice_mesh", ctypes.c_int, [vp, vp, vp]),
    ("qed3_lattice_set_spin_structure", ctypes.c_int, [vp, vp, vp]),
    ("qed3_lattice_permutation", ctypes.c_int, [vp, vp]),
    ("qed3_dirac_create", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.POINTER(vp)]),
    ("qed3_dirac_create_1f", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.POINTER(vp)]),
    ("qed3_dirac_destroy", ctypes.c_int, [vp]),
    ("qed3_dirac_set_links", ctypes.c_int, [vp, vp, ctypes.c_int, vp]),
    ("qed3_dirac_set_coefficients", ctypes.c_int, [vp, vp, vp]),
    ("qed3_dirac_apply", ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp]),
    ("qed3_field_bytes", ctypes.c_size_t, [vp, ctypes.c_int, ctypes.c_int]),
    ("qed3_field_import", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp]),
    ("qed3_field_export", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp]),
    ("qed3_dirac_apply_field", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp]),
    ("qed3_cg_solve", ctypes.c_int, [vp, vp, vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveReport), vp]),
    ("qed3_solver_last_report", ctypes.c_int, [vp, ctypes.POINTER(SolveReport)]),
    ("qed3_dirac_spectral_bounds", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_int, c_double_p, c_double_p,
                                                  c_int_p, vp]),
    ("qed3_bicgstab_solve", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.POINTER(SolveParams), ctypes.c_double,
                                           ctypes.POINTER(SolveReport), vp]),
    ("qed3_cg_solve_noalloc", ctypes.c_int, [vp, vp, vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveReport),
                                             vp]),
    ("qed3_plaquette", ctypes.c_int, [vp, vp, vp, c_double_p, vp]),
    ("qed3_gauge_action", ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int, c_double_p, vp]),
    ("qed3_gauge_force", ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp, vp]),
    ("qed3_fermion_force", ctypes.c_int, [vp, vp, vp, vp]),
    ("qed3_rng_create", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]),
    ("qed3_rng_destroy", ctypes.c_int, [vp]),
    ("qed3_rng_gaussian_links", ctypes.c_int, [vp, ctypes.c_double, vp]),
    ("qed3_rng_gaussian_spinor", ctypes.c_int, [vp, vp]),
    ("qed3_rng_z2_spinor", ctypes.c_int, [vp, vp]),
    ("qed3_point_source", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]),
    ("qed3_hmc_fermion", ctypes.c_int, [vp, vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, c_int_p, c_double_p, c_int_p, vp]),
    ("qed3_hmc_overlap", ctypes.c_int, [vp, vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, c_int_p, c_double_p, c_int_p,
                                        vp]),
    ("qed3_hmc_pure_gauge", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_int, ctypes.c_int, c_int_p, c_double_p, vp]),
    ("qed3_zolotarev", ctypes.c_int, [ctypes.c_double, ctypes.c_int, vp, vp, vp, vp, c_int_p]),
    ("qed3_overlap_create", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]),
    ("qed3_overlap_destroy", ctypes.c_int, [vp]),
    ("qed3_overlap_update", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]),
    ("qed3_overlap_info", ctypes.c_int, [vp, c_double_p, c_double_p, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("qed3_overlap_apply", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.POINTER(SolveReport),
                                          vp]),
    ("qed3_overlap_force", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.POINTER(SolveReport), vp]),
    ("qed3_overlap_solve", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                          ctypes.POINTER(SolveReport), vp]),
    ("qed3_overlap_solve2", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(SolveReport), vp]),
    ("qed3_overlap_project_low_modes", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                      ctypes.c_double, vp]),
    ("qed3_overlap_low_modes_info", ctypes.c_int, [vp, c_int_p, c_double_p, c_int_p, vp]),
    ("qed3_overlap_set_pole_solver", ctypes.c_int, [vp, ctypes.c_int]),
    ("qed3_overlap_set_mass", ctypes.c_int, [vp, ctypes.c_double]),
    ("qed3_multishift_solve", ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp, ctypes.c_double, ctypes.c_int, vp,
                                             ctypes.POINTER(ctypes.c_float), vp]),
    ("qed3_dirac_ext_create", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                             ctypes.POINTER(vp)]),
    ("qed3_dirac_ext_destroy", ctypes.c_int, [vp]),
    ("qed3_hmc_ext", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, c_int_p, c_double_p, c_int_p, vp]),
    ("qed3_dirac_ext_set_links", ctypes.c_int, [vp, vp, vp]),
    ("qed3_dirac_ext_apply", ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp]),
    ("qed3_dirac_ext_fermion_force", ctypes.c_int, [vp, vp, vp, vp]),
    ("qed3_dirac_ext_propagator", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                                 ctypes.POINTER(SolveParams), ctypes.POINTER(SolveReport), vp]),
    ("qed3_overlap_ext_create", ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(vp)]),
    ("qed3_overlap_ext_destroy", ctypes.c_int, [vp]),
    ("qed3_overlap_ext_update", ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               vp]),
    ("qed3_overlap_ext_info", ctypes.c_int, [vp, c_double_p, c_double_p, c_double_p, c_double_p]),
    ("qed3_overlap_ext_apply", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_double, c_int_p, vp]),
    ("qed3_overlap_ext_solve", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_int, ctypes.POINTER(SolveReport), vp]),
    ("qed3_overlap_ext_force", ctypes.c_int, [vp, vp, vp, ctypes.c_double, vp]),
    ("qed3_hmc_ext_overlap", ctypes.c_int, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, c_int_p,
                                            c_double_p, c_int_p, vp]),
    ("qed3_dirac_ext_cg_solve", ctypes.c_int, [vp, vp, vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveReport),
                                               vp]),
    ("qed3_ext_plaquettes", ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp, vp]),
    ("qed3_ext_gauge_action", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, c_double_p, vp]),
    ("qed3_ext_gauge_force", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, vp, vp]),
    ("qed3_ext_polyakov", ctypes.c_int, [vp, ctypes.c_int, vp, vp, c_double_p, vp]),
    ("qed3_batch_create", ctypes.c_int, [ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp)]),
    ("qed3_batch_create2", ctypes.c_int, [ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.POINTER(vp)]),
    ("qed3_batch_destroy", ctypes.c_int, [vp]),
    ("qed3_batch_config", ctypes.c_int, [vp, c_int_p, c_int_p, c_int_p]),
    ("qed3_batch_schedule", ctypes.c_int, [vp, c_int_p]),
    ("qed3_batch_solve", ctypes.c_int, [vp, vp, vp, vp, ctypes.POINTER(SolveParams), vp,
                                        ctypes.POINTER(ctypes.c_float), vp]),
    ("qed3_batch_set_shifts", ctypes.c_int, [vp, vp, ctypes.c_double, vp]),
    ("qed3_batch_launch", ctypes.c_int, [vp, vp, vp, ctypes.POINTER(SolveParams), vp]),
    ("qed3_batch_reports", ctypes.c_int, [vp, vp, vp]),
    ("qed3_lpc_create", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(vp)]),
    ("qed3_lpc_destroy", ctypes.c_int, [vp]),
    ("qed3_lpc_info", ctypes.c_int, [vp, c_int_p, c_int_p, c_int_p]),
    ("qed3_lpc_get_weights", ctypes.c_int, [vp, vp]),
    ("qed3_lpc_set_weights", ctypes.c_int, [vp, vp]),
    ("qed3_lpc_apply", ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp]),
    ("qed3_lpc_loss_grad", ctypes.c_int, [vp, vp, vp, ctypes.c_int, c_double_p, vp, vp]),
    ("qed3_lpc_collect", ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_uint, vp, ctypes.c_int, ctypes.c_int]),
    ("qed3_lpc_train", ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_uint, vp]),
    ("qed3_lpc_set_tensor_cores", ctypes.c_int, [vp, ctypes.c_int]),
    ("qed3_pcg_solve", ctypes.c_int, [vp, vp, vp, vp, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveReport),
                                      vp]),
]


def lib(build: bool = True):
    """Load (building first if needed) the in-tree CUDA library."""
    global _lib
    if _lib is None:
        if build:
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise Qed3Error(ERR_STATE, f"{LIB_PATH} is missing; run qed3_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        msg = lib().qed3_last_error_string().decode()
        raise Qed3Error(rc, msg)


def _ptr(t):
    """Device pointer of a torch tensor, or data pointer of a numpy array."""
    if isinstance(t, np.ndarray):
        return t.ctypes.data_as(vp)
    if t is None:
        return None
    return vp(t.data_ptr())


def _stream(stream):
    if stream is None:
        return None
    return vp(getattr(stream, "cuda_stream", stream))


class S2Trivalent:
    """Dual trivalent lattice of refinement n (S2Trivalent, src/both_3d/s2n_dual.h:49)."""

    def __init__(self, n_refine: int, _handle=None):
        self.n_refine = n_refine
        if _handle is None:
            h = vp()
            _check(lib().qed3_lattice_create(n_refine, ctypes.byref(h)))
        else:
            h = _handle
        self._h = h
        ns, nl, nf, ft = (ctypes.c_int() for _ in range(4))
        _check(lib().qed3_lattice_sizes(h, *(ctypes.byref(v) for v in (ns, nl, nf, ft))))
        self.n_sites, self.n_links, self.n_faces, self.face_total = ns.value, nl.value, nf.value, ft.value
        self._tables = None

    @classmethod
    def from_mesh(cls, vertices, triangles, links=None) -> "S2Trivalent":
        """The dual lattice of a caller's closed triangulation of the sphere, in the
        caller's numbering (dual site t = triangle t; links in the given (i<j) order,
        else lexicographic)."""
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        lk = None if links is None else np.ascontiguousarray(links, dtype=np.int32).reshape(-1, 2)
        h = vp()
        _check(lib().qed3_lattice_from_mesh(v.shape[0], _ptr(v), t.shape[0], _ptr(t),
                                            None if lk is None else _ptr(lk), ctypes.byref(h)))
        return cls(0, _handle=h)

    def mesh(self):
        """(vertices [n_faces, 3], triangles [n_sites, 3]) of the simplicial mesh."""
        v = np.zeros((self.n_faces, 3))
        t = np.zeros((self.n_sites, 3), np.int32)
        _check(lib().qed3_lattice_mesh(self._h, _ptr(v), _ptr(t)))
        return v, t

    def set_spin_structure(self, omega=None, alpha=None):
        """Use a caller's spin connection (omega per link, alpha per hop) for the
        operators created afterwards."""
        om = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64).reshape(self.n_links)
        al = None if alpha is None else np.ascontiguousarray(alpha, dtype=np.float64).reshape(self.n_sites * 3)
        _check(lib().qed3_lattice_set_spin_structure(self._h, None if om is None else _ptr(om),
                                                     None if al is None else _ptr(al)))
        self._tables = None

    @property
    def handle(self):
        return self._h

    def tables(self) -> dict:
        if self._tables is None:
            Ns, Nl, Nf, Ft = self.n_sites, self.n_links, self.n_faces, self.face_total
            t = dict(sites=np.zeros((Ns, 3)), nns=np.zeros((Ns, 3), np.int32), links=np.zeros((Nl, 2), np.int32),
                     simp_links=np.zeros((Nl, 2), np.int32), face_offsets=np.zeros(Nf + 1, np.int32),
                     face_sites=np.zeros(Ft, np.int32), ell=np.zeros(Nl), link_volume=np.zeros(Nl),
                     vols=np.zeros(Nf), omega=np.zeros(Nl), alpha=np.zeros((Ns, 3)), means=np.zeros(3))
            order = ["sites", "nns", "links", "simp_links", "face_offsets", "face_sites", "ell", "link_volume",
                     "vols", "omega", "alpha", "means"]
            _check(lib().qed3_lattice_tables(self._h, *(_ptr(t[k]) for k in order)))
            self._tables = t
        return self._tables

    def permutation(self) -> np.ndarray:
        p = np.zeros(self.n_sites, np.int32)
        _check(lib().qed3_lattice_permutation(self._h, _ptr(p)))
        return p

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_lattice_destroy(self._h)
            self._h = None


@dataclass
class Report:
    status: int
    iters: int
    reliable_updates: int
    true_rel_res: float
    ms: float


class DiracS2Dual:
    """Wilson-Dirac operator on the dual lattice with its device coefficients.

    Mirrors DiracS2Dual(lattice, m, r, M5) + DiracPf/DWDevice
    (src/both_3d/dirac_dual.h:63-106, src/both_3d/dirac_pf.h:4-125): the mass
    enters as M5, as in the reference where DiracS2Dual::m is unused.
    """

    def __init__(self, lattice: S2Trivalent, r: float = 1.0, M5: float = 0.0, one_flavor_mass: float | None = None):
        """one_flavor_mass = m: Dirac1fonS2's coefficients (src/dual/dirac.h:145-220)
        instead of DiracS2Dual's, with its real mass m."""
        self.lattice = lattice
        self.r, self.M5 = r, M5
        self.N = 2 * lattice.n_sites
        h = vp()
        if one_flavor_mass is None:
            _check(lib().qed3_dirac_create(lattice.handle, r, M5, ctypes.byref(h)))
        else:
            _check(lib().qed3_dirac_create_1f(lattice.handle, r, one_flavor_mass, M5, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def update(self, A, stream=None):
        """DWDevice::update(U): rebuild the hop blocks from link angles A[n_links]."""
        if isinstance(A, np.ndarray):
            A = np.ascontiguousarray(A, dtype=np.float64)
            _check(lib().qed3_dirac_set_links(self._h, _ptr(A), 0, _stream(stream)))
            self._sync(stream)
        else:
            _check(lib().qed3_dirac_set_links(self._h, _ptr(A), 1, _stream(stream)))

    def set_coefficients(self, hop: np.ndarray, diag: np.ndarray):
        hop = np.ascontiguousarray(hop, dtype=np.complex128).reshape(-1)
        diag = np.ascontiguousarray(diag, dtype=np.float64)
        _check(lib().qed3_dirac_set_coefficients(self._h, _ptr(hop), _ptr(diag)))

    def apply(self, out, inp, op: int = OP_D, stream=None):
        """LinOp::operator(): out = op(inp) on device complex128 tensors."""
        _check(lib().qed3_dirac_apply(self._h, op, _ptr(out), _ptr(inp), _stream(stream)))
        return out

    # -- device-internal fields ---------------------------------------------------
    def field_bytes(self, prec: int, nrhs: int = 1) -> int:
        return lib().qed3_field_bytes(self._h, prec, nrhs)

    def field_import(self, field, inp, prec: int, nrhs: int = 1, stream=None):
        _check(lib().qed3_field_import(self._h, prec, _ptr(field), _ptr(inp), nrhs, _stream(stream)))

    def field_export(self, out, field, prec: int, nrhs: int = 1, stream=None):
        _check(lib().qed3_field_export(self._h, prec, _ptr(out), _ptr(field), nrhs, _stream(stream)))

    def apply_field(self, out, inp, op: int, prec: int, nrhs: int = 1, stream=None):
        _check(lib().qed3_dirac_apply_field(self._h, op, prec, _ptr(out), _ptr(inp), nrhs, _stream(stream)))

    # -- solver ----------------------------------------------------------------------
    def solve(self, x, b, tol: float = 1e-10, maxiter: int = 100000, precision: int = PREC_F64,
              delta: float = 0.1, shift: float = 0.0, flags: int = 0, stream=None) -> Report:
        """CG on (D^dagger D + shift) x = b (MatPoly::solve); certified by the FP64 true residual."""
        p = SolveParams(tol, maxiter, precision, delta, shift, flags)
        r = SolveReport()
        rc = lib().qed3_cg_solve(self._h, _ptr(x), _ptr(b), ctypes.byref(p), ctypes.byref(r), _stream(stream))
        if rc not in (OK, ERR_NOCONV):
            _check(rc)
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def spectral_bounds(self, tol: float = 1e-10, maxsteps: int = 20000, stream=None):
        """Extremal eigenvalues of D^dag D by device Lanczos: (lambda_min, lambda_max, steps, converged)."""
        lo, hi, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        rc = lib().qed3_dirac_spectral_bounds(self._h, tol, maxsteps, ctypes.byref(lo), ctypes.byref(hi),
                                              ctypes.byref(st), _stream(stream))
        if rc not in (OK, ERR_NOCONV):
            _check(rc)
        return lo.value, hi.value, st.value, rc == OK

    def bicgstab(self, x, b, op: int = OP_D, tol: float = 1e-10, maxiter: int = 100000, shift: float = 0.0,
                 eps: float = 1e-8, stream=None) -> Report:
        """BiCGStab with restarts (MatPoly::bicgstab) on (op + shift) x = b, FP64."""
        p = SolveParams(tol, maxiter, PREC_F64, 0.1, shift, 0)
        r = SolveReport()
        rc = lib().qed3_bicgstab_solve(self._h, op, _ptr(x), _ptr(b), ctypes.byref(p), eps, ctypes.byref(r),
                                       _stream(stream))
        _check(rc)
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    @staticmethod
    def _sync(stream):
        import torch
        if torch.cuda.is_available():
            (stream or torch.cuda.current_stream()).synchronize()

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_dirac_destroy(self._h)
            self._h = None


# ---------------------------------------------------------------------------
# gauge side
# ---------------------------------------------------------------------------
def plaquette(lattice: S2Trivalent, A, theta=None, stream=None) -> float:
    """Plaquette angles into `theta` (device, optional); returns mean cos(theta)."""
    avg = ctypes.c_double()
    _check(lib().qed3_plaquette(lattice.handle, _ptr(A), _ptr(theta), ctypes.byref(avg), _stream(stream)))
    return avg.value


def gauge_action(lattice: S2Trivalent, A, beta: float, compact: bool = True, stream=None) -> float:
    S = ctypes.c_double()
    _check(lib().qed3_gauge_action(lattice.handle, _ptr(A), beta, int(compact), ctypes.byref(S), _stream(stream)))
    return S.value


def gauge_force(lattice: S2Trivalent, A, F, beta: float, compact: bool = True, exact: bool = True, stream=None):
    _check(lib().qed3_gauge_force(lattice.handle, _ptr(A), beta, int(compact), int(exact), _ptr(F), _stream(stream)))
    return F


def fermion_force(dirac: DiracS2Dual, eta, F, stream=None):
    _check(lib().qed3_fermion_force(dirac.handle, _ptr(eta), _ptr(F), _stream(stream)))
    return F


class ParallelRng:
    """ParallelRng2 (src/both/rng.h:76-125): seeded per-link and per-site engines.

    n_slices = Nt > 1: ParallelRngExt (src/both_3d/rng.h:89-121), engines
    [Nt][n_links] and [Nt][n_sites], the streams of S^2 x S^1 HMC."""

    def __init__(self, lattice: S2Trivalent, seed: int = 0, n_slices: int = 1):
        self.lattice = lattice
        self.n_slices = n_slices
        h = vp()
        _check(lib().qed3_rng_create(lattice.n_links * n_slices, lattice.n_sites * n_slices, seed,
                                     ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def gaussian_links(self, width: float = 1.0) -> np.ndarray:
        out = np.zeros(self.lattice.n_links * self.n_slices)
        _check(lib().qed3_rng_gaussian_links(self._h, width, _ptr(out)))
        return out

    def gaussian_spinor(self) -> np.ndarray:
        out = np.zeros(2 * self.lattice.n_sites * self.n_slices, np.complex128)
        _check(lib().qed3_rng_gaussian_spinor(self._h, _ptr(out)))
        return out

    def uniform(self) -> float:
        """One master-engine uniform draw (the Metropolis test's)."""
        u = ctypes.c_double()
        _check(lib().qed3_rng_uniform(self._h, ctypes.byref(u)))
        return u.value

    def save(self, path: str):
        """Checkpoint the streams (the reference's ParallelRngExt::ckpoint layout)."""
        _check(lib().qed3_rng_save(self._h, os.fsencode(path)))

    def load(self, path: str):
        _check(lib().qed3_rng_load(self._h, os.fsencode(path)))

    def z2_spinor(self) -> np.ndarray:
        """FermionVector::set_random: (z + i z')/sqrt(2 Ns), z from the site engines' dist_z2(1, 2)."""
        out = np.zeros(2 * self.lattice.n_sites * self.n_slices, dtype=np.complex128)
        _check(lib().qed3_rng_z2_spinor(self._h, _ptr(out)))
        return out

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_rng_destroy(self._h)
            self._h = None


def hmc_pure_gauge(lattice: S2Trivalent, rng: ParallelRng, A, beta: float, compact: bool = True,
                   exact: bool = True, tmax: float = 1.0, nsteps: int = 40, no_reject: bool = False, stream=None):
    """One HMCPureGauge trajectory in place on the device links A; returns (accepted, dH)."""
    acc = ctypes.c_int()
    dH = ctypes.c_double()
    _check(lib().qed3_hmc_pure_gauge(lattice.handle, rng.handle, _ptr(A), beta, int(compact), int(exact), tmax,
                                     nsteps, int(no_reject), ctypes.byref(acc), ctypes.byref(dH), _stream(stream)))
    return bool(acc.value), dH.value


def hmc_fermion(lattice: S2Trivalent, dirac: DiracS2Dual, rng: "ParallelRng", A, beta: float, compact: bool = True,
                exact: bool = True, tmax: float = 1.0, nsteps: int = 10, nsteps_inner: int = 10, tol: float = 1e-10,
                precision: int = PREC_F32, no_reject: bool = False, npf: int = 1,
                integrator: int = 0, stream=None):
    """One Wilson-fermion HMC trajectory on device links A (in place): HMC::run (npf = 1)
    or HMC2::run (npf pseudofermions) with ExplicitLeapfrogML (integrator
    INTEGRATOR_LEAPFROG_ML) or ExplicitLeapfrog (INTEGRATOR_LEAPFROG).  Returns
    (accepted, dH, cg_iterations)."""
    acc, dH, its = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    _check(lib().qed3_hmc_fermion(lattice.handle, dirac.handle, rng.handle, _ptr(A), beta, int(compact), int(exact),
                                  tmax, nsteps, nsteps_inner, npf, integrator, tol, precision, int(no_reject), ctypes.byref(acc),
                                  ctypes.byref(dH), ctypes.byref(its), _stream(stream)))
    return bool(acc.value), dH.value, its.value


def hmc_overlap(lattice: S2Trivalent, overlap: "Overlap", rng: "ParallelRng", A, beta: float, compact: bool = True,
                exact: bool = True, tmax: float = 1.0, nsteps: int = 10, nsteps_inner: int = 10, npf: int = 1,
                lambda_min: float = 0.0, lambda_max: float = 0.0, tol: float = 1e-10, tol_inner: float = 1e-12,
                no_reject: bool = False, integrator: int = 0, stream=None):
    """One overlap-fermion HMC trajectory (HMC2::run with Overlap fermions) on device
    links A, in place.  lambda_min = lambda_max = 0: the operator update recomputes
    the spectral bounds (Overlap::update); otherwise the bounds stay fixed.
    Returns (accepted, dH, outer_cg_iterations)."""
    acc, dH, its = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    _check(lib().qed3_hmc_overlap(lattice.handle, overlap._h, rng.handle, _ptr(A), beta, int(compact), int(exact),
                                  tmax, nsteps, nsteps_inner, npf, integrator, lambda_min, lambda_max, tol, tol_inner,
                                  int(no_reject), ctypes.byref(acc), ctypes.byref(dH), ctypes.byref(its),
                                  _stream(stream)))
    return bool(acc.value), dH.value, its.value


def thermalized_links(lattice: S2Trivalent, beta: float, seed: int, ntraj: int, init: str = "uniform",
                      device="cuda", compact: bool = True, nsteps: int = 40):
    """Seeded configuration: A ~ U[-pi, pi) (init="uniform") or 0.2 N(0,1)
    (init="gaussian", src/both/gauge.cu:157), then `ntraj` pure-gauge HMC
    trajectories (tmax=1, nsteps) at `beta`.  Returns (device links, acceptance)."""
    import torch

    rng = ParallelRng(lattice, seed)
    if init == "uniform":
        A0 = np.random.default_rng(seed).uniform(-np.pi, np.pi, lattice.n_links)
    else:
        A0 = rng.gaussian_links(0.2)
    A = torch.from_numpy(A0).to(device)
    acc = 0
    for _ in range(ntraj):
        a, _ = hmc_pure_gauge(lattice, rng, A, beta, compact, True, 1.0, nsteps)
        acc += a
    return A, acc / max(1, ntraj)


def multishift_solve(dirac: DiracS2Dual, x, b, shifts, tol: float = 1e-10, maxiter: int = 200000, stream=None):
    """x[m] = (D^dag D + shifts[m])^{-1} b in one Krylov space (FP64 multi-shift CG).
    x: device complex128 (nshifts, 2*n_sites); returns (reports, ms)."""
    sh = np.ascontiguousarray(shifts, dtype=np.float64)
    reps = (SolveReport * len(sh))()
    ms = ctypes.c_float()
    _check(lib().qed3_multishift_solve(dirac.handle, len(sh), _ptr(sh), _ptr(x), _ptr(b), tol, maxiter, reps,
                                       ctypes.byref(ms), _stream(stream)))
    return [Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms) for r in reps], ms.value


def point_source(lattice: S2Trivalent, x: int, s: int) -> np.ndarray:
    """FermionVector::set_pt_source (src/dual/valence.h:47-52): unit vector at (site x, spin s)."""
    out = np.zeros(2 * lattice.n_sites, dtype=np.complex128)
    _check(lib().qed3_point_source(lattice.n_sites, x, s, _ptr(out)))
    return out


def save_links(lattice: S2Trivalent, A, path: str):
    """Gauge checkpoint in the reference's GaugeExt::ckpoint layout (Nt = 1)."""
    h = np.ascontiguousarray(A.detach().cpu().numpy() if hasattr(A, "detach") else A, dtype=np.float64)
    _check(lib().qed3_links_save(lattice.handle, _ptr(h), os.fsencode(path)))


def load_links(lattice: S2Trivalent, path: str) -> np.ndarray:
    """Reads a GaugeExt checkpoint (Nt = 1); returns the host link angles."""
    A = np.zeros(lattice.n_links)
    t = ctypes.c_double()
    _check(lib().qed3_links_load(lattice.handle, _ptr(A), ctypes.byref(t), os.fsencode(path)))
    return A


def selftest_wait_timeout(spin_limit: int = 20000):
    """Run the bounded-wait self-test; returns (status, resident_timed_out, streaming_timed_out)."""
    a, b = ctypes.c_int(), ctypes.c_int()
    rc = lib().qed3_selftest_wait_timeout(spin_limit, ctypes.byref(a), ctypes.byref(b))
    return rc, bool(a.value), bool(b.value)


def zolotarev(k: float, n: int) -> dict:
    """Zolotarev coefficients of sign(x) on [k, 1] (Zolotarev, src/both_3d/overlap.h:7-116)."""
    size = n // 2 + 1
    c, cp, A, sc = np.zeros(size), np.zeros(size), np.zeros(size), np.zeros(4)
    sz = ctypes.c_int()
    _check(lib().qed3_zolotarev(k, n, _ptr(c), _ptr(cp), _ptr(A), _ptr(sc), ctypes.byref(sz)))
    return dict(c=c, cp=cp, A=A, M=sc[0], lambda_inv=sc[1], E=sc[2], C=sc[3], size=size, k=k, n=n)


# ---------------------------------------------------------------------------
# batched persistent solver
# ---------------------------------------------------------------------------
def ext_plaquettes(lattice: S2Trivalent, Nt: int, A, theta_s, theta_t, stream=None):
    """S^2 x S^1 spatial [Nt][n_faces] and temporal [Nt][n_links] plaquette angles (device)."""
    _check(lib().qed3_ext_plaquettes(lattice.handle, Nt, _ptr(A), _ptr(theta_s), _ptr(theta_t), _stream(stream)))


def ext_gauge_action(lattice: S2Trivalent, Nt: int, at: float, gsq: float, A, stream=None) -> float:
    S = ctypes.c_double()
    _check(lib().qed3_ext_gauge_action(lattice.handle, Nt, at, gsq, _ptr(A), ctypes.byref(S), _stream(stream)))
    return S.value


def ext_gauge_force(lattice: S2Trivalent, Nt: int, at: float, gsq: float, A, F, stream=None):
    _check(lib().qed3_ext_gauge_force(lattice.handle, Nt, at, gsq, _ptr(A), _ptr(F), _stream(stream)))
    return F


def ext_polyakov(lattice: S2Trivalent, Nt: int, A, P=None, stream=None):
    """Polyakov loop per site into P (device complex128, optional); returns its mean."""
    avg = (ctypes.c_double * 2)()
    _check(lib().qed3_ext_polyakov(lattice.handle, Nt, _ptr(A), _ptr(P), avg, _stream(stream)))
    return complex(avg[0], avg[1])


class DiracExt:
    """S^2 x S^1 Wilson-Dirac operator with Nt time slices (DiracExt, src/both_3d/dirac_ext.h:6-334).

    Vectors: device complex128 of Nt * 2 * n_sites (slice-major); links: device
    float64 [Nt * n_links spatial, then Nt * n_sites temporal]."""

    def __init__(self, lattice: S2Trivalent, r: float = 1.0, M5: float = 0.0, Nt: int = 1, at: float = 1.0):
        self.lattice, self.r, self.M5, self.Nt, self.at = lattice, r, M5, Nt, at
        self.N = 2 * lattice.n_sites * Nt
        h = vp()
        _check(lib().qed3_dirac_ext_create(lattice.handle, r, M5, Nt, at, ctypes.byref(h)))
        self._h = h

    def update(self, A, stream=None):
        _check(lib().qed3_dirac_ext_set_links(self._h, _ptr(A), _stream(stream)))

    def apply(self, out, inp, op: int = OP_D, stream=None):
        _check(lib().qed3_dirac_ext_apply(self._h, op, _ptr(out), _ptr(inp), _stream(stream)))
        return out

    def fermion_force(self, eta, F, stream=None):
        """F (device, link layout) = -2 Re <D eta, dD/dA eta>."""
        _check(lib().qed3_dirac_ext_fermion_force(self._h, _ptr(eta), _ptr(F), _stream(stream)))
        return F

    def solve(self, x, b, tol: float = 1e-10, maxiter: int = 100000, shift: float = 0.0, precision: int = PREC_F64,
              delta: float = 0.1, stream=None) -> Report:
        """CG on D^dag D + shift; precision PREC_F32: FP32 iterations with FP64
        reliable updates (same FP64 certificate)."""
        p = SolveParams(tol, maxiter, precision, delta, shift, 0)
        r = SolveReport()
        _check(lib().qed3_dirac_ext_cg_solve(self._h, _ptr(x), _ptr(b), ctypes.byref(p), ctypes.byref(r),
                                             _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def propagator(self, sink, s: int = 0, ix: int = 0, spin: int = 0, tol: float = 1e-10, dagger: bool = False,
                   precision: int = PREC_F64, stream=None) -> Report:
        """sink = D^{-1} (point source at slice s, site ix, spin), prop.cu's
        (D^dag D)^{-1} D^dag src solve; dagger: D^{-dag} (IS_DAGGER)."""
        p = SolveParams(tol, 0, precision, 0.1, 0.0, 0)
        r = SolveReport()
        _check(lib().qed3_dirac_ext_propagator(self._h, s, ix, spin, int(dagger), _ptr(sink), ctypes.byref(p), ctypes.byref(r),
                                               _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_dirac_ext_destroy(self._h)
            self._h = None


class OverlapExt:
    """Overlap<DiracExt>: the overlap operator of the S^2 x S^1 Wilson operator
    (src/both_3d/overlap.h:137-390), all poles in one FP64 multi-shift CG."""

    def __init__(self, dirac: DiracExt, order: int = 21):
        self.dirac = dirac
        h = vp()
        _check(lib().qed3_overlap_ext_create(dirac._h, order, ctypes.byref(h)))
        self._h = h

    def update(self, lambda_min: float = 0.0, lambda_max: float = 0.0, tol: float = 1e-10, margin: float = 1e-6,
               stream=None):
        _check(lib().qed3_overlap_ext_update(self._h, lambda_min, lambda_max, tol, margin, _stream(stream)))

    def info(self) -> dict:
        a, b, k, dl = (ctypes.c_double() for _ in range(4))
        _check(lib().qed3_overlap_ext_info(self._h, *(ctypes.byref(v) for v in (a, b, k, dl))))
        return dict(lambda_min=a.value, lambda_max=b.value, k=k.value, delta=dl.value)

    def apply(self, out, inp, op: int = OP_D, tol_inner: float = 1e-12, stream=None) -> int:
        it = ctypes.c_int()
        _check(lib().qed3_overlap_ext_apply(self._h, op, _ptr(out), _ptr(inp), tol_inner, ctypes.byref(it),
                                            _stream(stream)))
        return it.value

    def solve(self, x, b, tol: float = 1e-10, tol_inner: float = 1e-12, maxiter: int = 100000,
              propagator: bool = False, stream=None) -> Report:
        r = SolveReport()
        _check(lib().qed3_overlap_ext_solve(self._h, _ptr(x), _ptr(b), tol, tol_inner, maxiter, int(propagator),
                                            ctypes.byref(r), _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def force(self, eta, F, tol_inner: float = 1e-12, stream=None):
        """F = -2 d/dA Re<eta, D_ov eta> (device, S^2 x S^1 link layout)."""
        _check(lib().qed3_overlap_ext_force(self._h, _ptr(eta), _ptr(F), tol_inner, _stream(stream)))
        return F

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_overlap_ext_destroy(self._h)
            self._h = None


def hmc_ext_overlap(overlap: OverlapExt, rng: ParallelRng, A, gsq: float, tmax: float = 1.0, nsteps: int = 10,
                    nsteps_inner: int = 10, npf: int = 1, integrator: int = 0, tol: float = 1e-10,
                    tol_inner: float = 1e-12, lambda_min: float = 0.0, lambda_max: float = 0.0,
                    no_reject: bool = False, stream=None):
    """One S^2 x S^1 HMC trajectory with Overlap<DiracExt> pseudofermions (the
    reference's IS_OVERLAP hmc.cu); bounds fixed or recomputed at every update."""
    acc, dH, its = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    _check(lib().qed3_hmc_ext_overlap(overlap._h, rng.handle, _ptr(A), overlap.dirac.at, gsq, tmax, nsteps,
                                      nsteps_inner, npf, integrator, tol, tol_inner, lambda_min, lambda_max,
                                      int(no_reject), ctypes.byref(acc), ctypes.byref(dH), ctypes.byref(its),
                                      _stream(stream)))
    return bool(acc.value), dH.value, its.value


def hmc_ext(dirac: DiracExt, rng: ParallelRng, A, gsq: float, tmax: float = 1.0, nsteps: int = 10,
            nsteps_inner: int = 10, npf: int = 1, integrator: int = 0, tol: float = 1e-10, no_reject: bool = False,
            precision: int = PREC_F64, stream=None):
    """One S^2 x S^1 HMC trajectory (HMC2::run with U1WilsonExt(at, gsq) and npf
    DiracExt pseudofermions) on device links A, in place; rng =
    ParallelRng(lattice, seed, n_slices=Nt).  Returns (accepted, dH, cg_iterations)."""
    acc, dH, its = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    _check(lib().qed3_hmc_ext(dirac._h, rng.handle, _ptr(A), dirac.at, gsq, tmax, nsteps, nsteps_inner, npf,
                              integrator, tol, precision, int(no_reject), ctypes.byref(acc), ctypes.byref(dH),
                              ctypes.byref(its), _stream(stream)))
    return bool(acc.value), dH.value, its.value


class Batch:
    """Several CG systems (lattices, right-hand sides, shifts) in one persistent launch.

    systems: list of (DiracS2Dual, nrhs).  rhs_tile (1, 2, 4, 8: right-hand
    sides sharing each stencil read), threads (128, 256) and schedule
    (BATCH_STATIC: a fixed range of blocks per system; BATCH_DYNAMIC: tiles of
    `threads` sites handed to free blocks at every CG step) = 0 let the built-in
    autotuner choose."""

    def __init__(self, systems, precision: int = PREC_F32, rhs_tile: int = 0, threads: int = 0, schedule: int = 0):
        self.systems = list(systems)
        n = len(self.systems)
        ops = (vp * n)(*[s[0].handle for s in self.systems])
        nr = (ctypes.c_int * n)(*[int(s[1]) for s in self.systems])
        h = vp()
        _check(lib().qed3_batch_create2(n, ops, nr, precision, rhs_tile, threads, schedule, ctypes.byref(h)))
        self._h = h
        R, T, B, S = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().qed3_batch_config(h, ctypes.byref(R), ctypes.byref(T), ctypes.byref(B)))
        _check(lib().qed3_batch_schedule(h, ctypes.byref(S)))
        self.rhs_tile, self.threads, self.blocks, self.schedule = R.value, T.value, B.value, S.value

    def solve(self, xs, bs, shifts=None, tol: float = 1e-10, maxiter: int = 100000, precision: int = PREC_F32,
              delta: float = 0.1, stream=None):
        """xs[u], bs[u]: device complex128 tensors of shape (nrhs_u, 2*n_sites) (or flat)."""
        n = len(self.systems)
        X = (vp * n)(*[x.data_ptr() for x in xs])
        B = (vp * n)(*[b.data_ptr() for b in bs])
        keep = []
        if shifts is not None:
            arrs = [np.ascontiguousarray(s, dtype=np.float64) if s is not None else None for s in shifts]
            keep = arrs
            S = (vp * n)(*[(a.ctypes.data if a is not None else None) for a in arrs])
        else:
            S = None
        total = sum(int(s[1]) for s in self.systems)
        reps = (SolveReport * total)()
        p = SolveParams(tol, maxiter, precision, delta, 0.0, 0)
        ms = ctypes.c_float()
        rc = lib().qed3_batch_solve(self._h, X, B, S, ctypes.byref(p), reps, ctypes.byref(ms), _stream(stream))
        del keep
        if rc not in (OK, ERR_NOCONV):
            _check(rc)
        return [Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms) for r in reps], ms.value

    # ---- the same solve in three calls, for CUDA-graph capture ----
    def set_shifts(self, shifts=None, shift: float = 0.0, stream=None):
        """Store the shifts on the device (only copies when they changed; must
        precede a capture)."""
        n = len(self.systems)
        arrs = [np.ascontiguousarray(s, dtype=np.float64) if s is not None else None for s in (shifts or [None] * n)]
        S = (vp * n)(*[(a.ctypes.data if a is not None else None) for a in arrs])
        _check(lib().qed3_batch_set_shifts(self._h, S if shifts is not None else None, shift, _stream(stream)))

    def launch(self, xs, bs, tol: float = 1e-10, maxiter: int = 100000, delta: float = 0.1, broadcast: bool = False,
               stream=None):
        """Enqueue one solve with no host synchronisation: capturable with
        torch.cuda.graph (pass the capturing stream)."""
        n = len(self.systems)
        self._X = (vp * n)(*[x.data_ptr() for x in xs])
        self._B = (vp * n)(*[b.data_ptr() for b in bs])
        p = SolveParams(tol, maxiter, PREC_F32, delta, 0.0, SOLVE_BCAST_B if broadcast else 0)
        _check(lib().qed3_batch_launch(self._h, self._X, self._B, ctypes.byref(p), _stream(stream)))

    def reports(self, stream=None):
        """Wait for the stream and report the last completed launch."""
        total = sum(int(s[1]) for s in self.systems)
        reps = (SolveReport * total)()
        rc = lib().qed3_batch_reports(self._h, reps, _stream(stream))
        if rc not in (OK, ERR_NOCONV):
            _check(rc)
        return [Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms) for r in reps]

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_batch_destroy(self._h)
            self._h = None


class Overlap:
    """Overlap operator on top of a DiracS2Dual (Overlap<WilsonDirac>, src/both_3d/overlap.h:137).

    update(lmin, lmax): Zolotarev range [lmin/lmax, 1]; omit both to estimate
    them on the device with the reference's power iterations."""

    def __init__(self, dirac: DiracS2Dual, order: int = 21, precision: int = PREC_F32):
        self.dirac = dirac
        self.order = order
        h = vp()
        _check(lib().qed3_overlap_create(dirac.handle, order, precision, ctypes.byref(h)))
        self._h = h

    def update_lanczos(self, tol: float = 1e-10, margin: float = 1e-6, maxsteps: int = 20000, stream=None):
        """Spectral bounds from device Lanczos on D^dag D (no solves), widened by
        `margin` (relative) on each side, then the Zolotarev update."""
        lo, hi, steps, ok = self.dirac.spectral_bounds(tol, maxsteps, stream)
        if not ok:
            raise Qed3Error(ERR_NOCONV, f"Lanczos did not converge in {steps} steps")
        return self.update(np.sqrt(lo) * (1.0 - margin), np.sqrt(hi) * (1.0 + margin), stream=stream)

    def update(self, lambda_min: float = 0.0, lambda_max: float = 0.0, tol_outer: float = 1e-8, stream=None):
        _check(lib().qed3_overlap_update(self._h, lambda_min, lambda_max, tol_outer, _stream(stream)))
        return self.info()

    def info(self) -> dict:
        a, b, k, dl = (ctypes.c_double() for _ in range(4))
        np_, nh = ctypes.c_int(), ctypes.c_int()
        _check(lib().qed3_overlap_info(self._h, *(ctypes.byref(v) for v in (a, b, k, dl, np_, nh))))
        return dict(lambda_min=a.value, lambda_max=b.value, k=k.value, delta=dl.value, npoles=np_.value,
                    npoles_fp64=nh.value)

    def apply(self, out, inp, op: int = OP_D, tol_inner: float = 1e-10, stream=None) -> Report:
        r = SolveReport()
        _check(lib().qed3_overlap_apply(self._h, op, _ptr(out), _ptr(inp), tol_inner, ctypes.byref(r),
                                        _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def force(self, F, eta, tol_inner: float = 1e-10, stream=None) -> Report:
        """F[l] = -2 d/dA_l Re<eta, D_ov eta> for all links (Overlap::grad_deviceAsyncLaunch)."""
        r = SolveReport()
        _check(lib().qed3_overlap_force(self._h, _ptr(eta), _ptr(F), tol_inner, ctypes.byref(r), _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def solve(self, x, b, tol: float = 1e-10, tol_inner: float = 1e-12, maxiter: int = 10000, flags: int = 0,
              stream=None) -> Report:
        """Outer CG on D_ov^dag D_ov x = b; true_rel_res recomputed after convergence.
        flags: OVSOLVE_CHIRAL (chirality sectors, one pole solve per iteration)."""
        r = SolveReport()
        if flags:
            _check(lib().qed3_overlap_solve2(self._h, _ptr(x), _ptr(b), tol, tol_inner, maxiter, flags,
                                             ctypes.byref(r), _stream(stream)))
        else:
            _check(lib().qed3_overlap_solve(self._h, _ptr(x), _ptr(b), tol, tol_inner, maxiter, ctypes.byref(r),
                                            _stream(stream)))
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def project_low_modes(self, nev: int, tol: float = 1e-13, maxsteps: int = 6000, margin: float = 1e-3,
                          stream=None) -> dict:
        """Treat the nev eigenmodes of gamma5 D_W nearest zero exactly in the sign
        function; the Zolotarev range then starts above them (nev = 0: off)."""
        _check(lib().qed3_overlap_project_low_modes(self._h, nev, tol, maxsteps, margin, _stream(stream)))
        return self.low_modes_info()

    def set_mass(self, mass: float):
        """D(m) = (1 - m/2) D_ov + m for apply and the outer solves (0: massless)."""
        _check(lib().qed3_overlap_set_mass(self._h, mass))

    def set_pole_solver(self, mode: int):
        """POLES_MULTISHIFT (FP64 multi-shift CG, default) or POLES_BATCHED
        (one mixed-precision CG per pole in one batched launch)."""
        _check(lib().qed3_overlap_set_pole_solver(self._h, mode))

    def low_modes_info(self) -> dict:
        n, res, steps = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        _check(lib().qed3_overlap_low_modes_info(self._h, ctypes.byref(n), ctypes.byref(res), ctypes.byref(steps),
                                                 None))
        mu = np.zeros(max(1, n.value))
        _check(lib().qed3_overlap_low_modes_info(self._h, None, None, None, _ptr(mu)))
        return dict(nev=n.value, max_residual=res.value, lanczos_steps=steps.value, mu=mu[:n.value],
                    **self.info())

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_overlap_destroy(self._h)
            self._h = None


class LearnedPreconditioner:
    """Gauge-covariant learned preconditioner N = a^2 I + G^dag G (no counterpart
    in the reference, whose solvers are unpreconditioned CG,
    src/both_3d/cg_cuda.h).  Trained on the GPU on (residual, error) pairs from
    the solver's own iterates; applied block-locally inside the persistent
    preconditioned CG (``solve``)."""

    def __init__(self, dirac: DiracS2Dual, channels: int = 16, layers: int = 2, seed: int = 0):
        self.dirac = dirac
        self.channels, self.layers = channels, layers
        h = vp()
        _check(lib().qed3_lpc_create(dirac.handle, channels, layers, seed, ctypes.byref(h)))
        self._h = h

    def set_tensor_cores(self, enable: bool):
        """16 -> 16 channel mixing on the tensor cores (BF16 operands, FP32 accumulate) or FP32 CUDA cores."""
        _check(lib().qed3_lpc_set_tensor_cores(self._h, 1 if enable else 0))

    def info(self) -> dict:
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().qed3_lpc_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return dict(nparams=a.value, block_sites=b.value, npairs=c.value)

    def get_weights(self) -> np.ndarray:
        w = np.zeros(2 * self.info()["nparams"])
        _check(lib().qed3_lpc_get_weights(self._h, _ptr(w)))
        return w.view(np.complex128)

    def set_weights(self, w):
        w = np.ascontiguousarray(np.asarray(w, dtype=np.complex128))
        _check(lib().qed3_lpc_set_weights(self._h, _ptr(w)))

    def apply(self, z, r, nrhs: int = 1, form: int = 0, stream=None):
        """z = N r; device complex128, reference order, nrhs vectors back to back."""
        _check(lib().qed3_lpc_apply(self._h, form, _ptr(z), _ptr(r), nrhs, _stream(stream)))
        return z

    def loss_grad(self, r, e, nrhs: int = 1, stream=None):
        loss = ctypes.c_double()
        g = np.zeros(2 * self.info()["nparams"])
        _check(lib().qed3_lpc_loss_grad(self._h, _ptr(r), _ptr(e), nrhs, ctypes.byref(loss), _ptr(g),
                                        _stream(stream)))
        return loss.value, g.view(np.complex128)

    def collect(self, dirac: DiracS2Dual, nsrc: int, seed: int, snapshots=(0, 5, 20, 60, 150),
                precision: int = PREC_F32):
        snaps = np.ascontiguousarray(snapshots, dtype=np.int32)
        _check(lib().qed3_lpc_collect(self._h, dirac.handle, nsrc, seed, _ptr(snaps), len(snaps), precision))

    def train(self, steps: int, batch: int = 8, lr: float = 3e-3, seed: int = 0) -> np.ndarray:
        hist = np.zeros(max(steps, 1))
        _check(lib().qed3_lpc_train(self._h, steps, batch, lr, seed, _ptr(hist)))
        return hist[:steps]

    def solve(self, dirac: DiracS2Dual, x, b, tol: float = 1e-10, maxiter: int = 100000,
              precision: int = PREC_F32, delta: float = 0.1, shift: float = 0.0, flexible: bool = False,
              pipelined: bool = False, stream=None) -> Report:
        """Preconditioned CG on (D^dag D + shift) x = b; FP64 true-residual certificate.
        flexible: Polak-Ribiere beta (flexible CG), robust to a preconditioner that is
        not exactly linear or hermitian."""
        flags = (SOLVE_FLEXIBLE if flexible else 0) | (SOLVE_PIPELINED if pipelined else 0)
        p = SolveParams(tol, maxiter, precision, delta, shift, flags)
        r = SolveReport()
        rc = lib().qed3_pcg_solve(dirac.handle, self._h, _ptr(x), _ptr(b), ctypes.byref(p), ctypes.byref(r),
                                  _stream(stream))
        if rc not in (OK, ERR_NOCONV):
            _check(rc)
        return Report(r.status, r.iters, r.reliable_updates, r.true_rel_res, r.ms)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.qed3_lpc_destroy(self._h)
            self._h = None
