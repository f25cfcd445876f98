"""ctypes front end of the oracle's C restatement (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  Each wrapper names the reference function it restates;
the C file cites the reference lines.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None
_lapack_ok = None

dp = C.POINTER(C.c_double)
lp = C.POINTER(C.c_long)


class Rng(C.Structure):
    """State of filter/rand.c:28-66 ran_nrc (its statics made explicit)."""

    _fields_ = [("idum", C.c_long), ("idum2", C.c_long), ("iy", C.c_long),
                ("iv", C.c_long * 32)]


class Timing(C.Structure):
    _fields_ = [("energy_range_s", C.c_double), ("filter_s", C.c_double),
                ("ortho_s", C.c_double), ("hmat_s", C.c_double), ("sigma_s", C.c_double),
                ("iters", C.c_long), ("mkept", C.c_long), ("emax", C.c_double),
                ("dE", C.c_double), ("dt", C.c_double)]


def _p(a):
    return a.ctypes.data_as(dp)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        L.orc_rng_next.restype = C.c_double
        L.orc_box_half.restype = C.c_double
        L.orc_form_factor.restype = C.c_double
        L.orc_ctx_create.restype = C.c_void_p
        L.orc_ctx_create.argtypes = [C.c_long, C.c_long, C.c_long, dp, dp, C.c_double]
        L.orc_ctx_destroy.argtypes = [C.c_void_p]
        L.orc_hamiltonian.argtypes = [C.c_void_p, dp, dp]
        L.orc_hnorm.argtypes = [C.c_void_p, dp, dp, C.c_double, C.c_double, C.c_double]
        L.orc_filter_cycle.argtypes = [C.c_void_p, dp, dp, dp, C.c_long, C.c_long, C.c_double,
                                       C.c_double, dp]
        L.orc_energy_all.argtypes = [C.c_void_p, dp, C.c_long, dp]
        L.orc_energy_range.argtypes = [C.c_void_p, C.c_double, dp, dp]
        L.orc_energy_range.restype = C.c_long
        L.orc_portho.restype = C.c_long
        L.orc_portho.argtypes = [dp, C.c_long, C.c_long, dp]
        L.orc_hmat.argtypes = [C.c_void_p, dp, C.c_long, dp]
        L.orc_sigma.argtypes = [C.c_void_p, dp, C.c_long, dp]
        L.orc_pipeline.restype = C.c_long
        L.orc_pipeline.argtypes = [C.c_void_p, C.c_long, C.c_long, C.c_long, dp, C.c_double,
                                   C.c_double, dp, dp, dp, dp, C.c_int, C.c_int,
                                   C.POINTER(Timing)]
        L.orc_lapack_load.argtypes = [C.c_char_p]
        L.orc_filter_batch.restype = C.c_double
        L.orc_filter_batch.argtypes = [C.c_void_p, C.c_long, dp, dp, dp, C.c_long, C.c_long,
                                       C.c_double, C.c_double, dp, C.c_int]
        _lib = L
    return _lib


def lapack_available():
    global _lapack_ok
    if _lapack_ok is None:
        path = build_oracle.openblas_path()
        _lapack_ok = bool(path) and lib().orc_lapack_load(path.encode()) == 0
    return _lapack_ok


# ---- random numbers ---------------------------------------------------------
def rng(idum):
    r = Rng()
    lib().orc_rng_seed(C.byref(r), C.c_long(idum))
    return r


def uniforms(r, n):
    f = lib().orc_rng_next
    return np.array([f(C.byref(r)) for _ in range(n)])


def init_psi(r, ngrid, dv):
    """filter/init.c:236-251 init_psi, real part (the imaginary part is zero)."""
    out = np.empty(ngrid)
    lib().orc_init_psi(C.byref(r), C.c_long(ngrid), C.c_double(dv), _p(out))
    return out


def start_states(idum, ns, ngrid, dv):
    """filter/main.c:82-89: ns consecutive init_psi draws from one seed."""
    r = rng(idum)
    return np.stack([init_psi(r, ngrid, dv) for _ in range(ns)])


def normalize_all(psi, dv):
    """filter/norm.c:40-54 on [m, ngrid] real states (returns a copy)."""
    psi = np.ascontiguousarray(psi, dtype=np.float64).copy()
    lib().orc_normalize_all(_p(psi), C.c_double(dv), C.c_long(psi.shape[0]),
                            C.c_long(psi.shape[1]))
    return psi


# ---- set-up ----------------------------------------------------------------
def ksqr(nx, ny, nz, dx, dy, dz, ekinmax=10.0):
    out = np.empty(nx * ny * nz)
    lib().orc_ksqr(C.c_long(nx), C.c_long(ny), C.c_long(nz), C.c_double(dx), C.c_double(dy),
                   C.c_double(dz), C.c_double(ekinmax), _p(out))
    return out


def box_half(r):
    r = np.ascontiguousarray(r, dtype=np.float64)
    return lib().orc_box_half(_p(r), C.c_long(len(r)))


def center_atoms(rx, ry, rz):
    rx, ry, rz = (np.ascontiguousarray(a, dtype=np.float64).copy() for a in (rx, ry, rz))
    lib().orc_center_atoms(C.c_long(len(rx)), _p(rx), _p(ry), _p(rz))
    return rx, ry, rz


def shift_table(v):
    v = np.ascontiguousarray(v, dtype=np.float64).copy()
    lib().orc_shift_table(_p(v), C.c_long(len(v)))
    return v


def vbuild(rx, ry, rz, types, tab_r, tab_v, tab_n, dims, mins, steps, scale=None):
    """filter/init.c:157-182: tab_r/tab_v are [ntype, stride] arrays."""
    nx, ny, nz = dims
    tab_r = np.ascontiguousarray(tab_r, dtype=np.float64)
    tab_v = np.ascontiguousarray(tab_v, dtype=np.float64)
    tab_n = np.ascontiguousarray(tab_n, dtype=np.int64)
    types = np.ascontiguousarray(types, dtype=np.int64)
    rx, ry, rz = (np.ascontiguousarray(a, dtype=np.float64) for a in (rx, ry, rz))
    sc = None if scale is None else np.ascontiguousarray(scale, dtype=np.float64)
    out = np.empty(nx * ny * nz)
    lib().orc_vbuild(C.c_long(len(rx)), _p(rx), _p(ry), _p(rz),
                     types.ctypes.data_as(lp), None if sc is None else _p(sc), _p(tab_r),
                     _p(tab_v), tab_n.ctypes.data_as(lp), C.c_long(tab_r.shape[1]),
                     C.c_long(nx), C.c_long(ny), C.c_long(nz), *[C.c_double(v) for v in mins],
                     *[C.c_double(v) for v in steps], _p(out))
    return out


def form_factor_table(a, vol_per_atom):
    a = np.ascontiguousarray(a, dtype=np.float64)
    r = np.empty(1024)
    v = np.empty(1024)
    lib().orc_form_factor_table(_p(a), C.c_double(vol_per_atom), _p(r), _p(v))
    return r, v


# ---- Newton coefficients ----------------------------------------------------
def leja_points(nc):
    zr = np.empty(nc)
    zi = np.empty(nc)
    lib().orc_leja_points(C.c_long(nc), _p(zr), _p(zi))
    return zr, zi


def coefficients(el, nc, dE, vmin, dt):
    """filter/coeff.c:16-63: returns (an_re [ms, nc], an_im [ms, nc], zn [nc])."""
    el = np.ascontiguousarray(el, dtype=np.float64)
    ms = len(el)
    ar = np.empty((ms, nc))
    ai = np.empty((ms, nc))
    zn = np.empty(nc)
    lib().orc_coefficients(C.c_long(ms), C.c_long(nc), C.c_double(dE), C.c_double(vmin),
                           C.c_double(dt), _p(el), _p(ar), _p(ai), _p(zn))
    return ar, ai, zn


# ---- Hamiltonian context ----------------------------------------------------
class Context:
    """Grid + potential + k^2 of one system (the reference's potl/ksqr pair)."""

    def __init__(self, dims, potl, ksqr_arr, dv):
        self.nx, self.ny, self.nz = dims
        self.ngrid = self.nx * self.ny * self.nz
        self.potl = np.ascontiguousarray(potl, dtype=np.float64)
        self.ksqr = np.ascontiguousarray(ksqr_arr, dtype=np.float64)
        self.dv = float(dv)
        self.h = lib().orc_ctx_create(self.nx, self.ny, self.nz, _p(self.potl), _p(self.ksqr),
                                      self.dv)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_ctx_destroy(self.h)
            self.h = None

    def hamiltonian(self, psi):
        """filter/hamiltonian.c:11-23 on complex psi (ngrid,) complex128."""
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        out = np.empty_like(psi)
        lib().orc_hamiltonian(self.h, psi.ctypes.data_as(dp), out.ctypes.data_as(dp))
        return out

    def hnorm(self, psim1, dE_1, vmin, zm1):
        psim1 = np.ascontiguousarray(psim1, dtype=np.complex128)
        out = np.empty_like(psim1)
        lib().orc_hnorm(self.h, psim1.ctypes.data_as(dp), out.ctypes.data_as(dp), dE_1, vmin,
                        zm1)
        return out

    def filter_cycle(self, start, an_re, zn, dE_1, vmin):
        """filter/filter.c:59-83 for one real start state -> [ms, ngrid]."""
        an_re = np.ascontiguousarray(an_re, dtype=np.float64)
        ms, nc = an_re.shape
        start = np.ascontiguousarray(start, dtype=np.float64)
        zn = np.ascontiguousarray(zn, dtype=np.float64)
        out = np.empty((ms, self.ngrid))
        lib().orc_filter_cycle(self.h, _p(start), _p(an_re), _p(zn), ms, nc, dE_1, vmin,
                               _p(out))
        return out

    def filter_batch(self, start, an_re, zn, dE_1, vmin, nthreads=0):
        """filter/main.c:92-98: the cycles of [ns, N] start states on OpenMP
        threads; returns (out [ns, ms, N], wall seconds)."""
        start = np.ascontiguousarray(start, dtype=np.float64)
        an_re = np.ascontiguousarray(an_re, dtype=np.float64)
        zn = np.ascontiguousarray(zn, dtype=np.float64)
        ms, nc = an_re.shape
        out = np.empty((start.shape[0], ms, self.ngrid))
        sec = lib().orc_filter_batch(self.h, start.shape[0], _p(start), _p(an_re), _p(zn), ms,
                                     nc, dE_1, vmin, _p(out), nthreads)
        return out, sec

    def energy_all(self, psi0):
        psi0 = np.ascontiguousarray(psi0, dtype=np.float64)
        ene = np.empty(psi0.shape[0])
        lib().orc_energy_all(self.h, _p(psi0), psi0.shape[0], _p(ene))
        return ene

    def energy_range(self, vmin):
        emax = C.c_double()
        dE = C.c_double()
        it = lib().orc_energy_range(self.h, vmin, C.byref(emax), C.byref(dE))
        return emax.value, dE.value, it

    def portho(self, psi):
        if not lapack_available():
            raise RuntimeError("LAPACK (ILP64 OpenBLAS) not found for the oracle")
        psi = np.ascontiguousarray(psi, dtype=np.float64).copy()
        sv = np.empty(psi.shape[0])
        k = lib().orc_portho(_p(psi), self.ngrid, psi.shape[0], _p(sv))
        return psi, k, sv

    def hmat(self, psi):
        if not lapack_available():
            raise RuntimeError("LAPACK (ILP64 OpenBLAS) not found for the oracle")
        psi = np.ascontiguousarray(psi, dtype=np.float64).copy()
        ev = np.empty(psi.shape[0])
        rc = lib().orc_hmat(self.h, _p(psi), psi.shape[0], _p(ev))
        if rc != 0:
            raise RuntimeError("dsyev failed")
        return psi, ev

    def sigma(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        s = np.empty(psi.shape[0])
        lib().orc_sigma(self.h, _p(psi), psi.shape[0], _p(s))
        return s

    def pipeline(self, start, el, nc, vmin, dE=0.0, nthreads=0, subspace=True):
        """filter/main.c:64-142 with given start states; returns a dict."""
        if subspace and not lapack_available():
            raise RuntimeError("LAPACK (ILP64 OpenBLAS) not found for the oracle")
        start = np.ascontiguousarray(start, dtype=np.float64)
        el = np.ascontiguousarray(el, dtype=np.float64)
        ns, ms = start.shape[0], len(el)
        psitot = np.empty((ns * ms, self.ngrid))
        ev = np.zeros(ns * ms)
        sg = np.zeros(ns * ms)
        t = Timing()
        mk = lib().orc_pipeline(self.h, ns, ms, nc, _p(el), vmin, dE, _p(start), _p(psitot),
                                _p(ev), _p(sg), nthreads, 1 if subspace else 0, C.byref(t))
        return {"psi": psitot[:mk], "eval": ev[:mk], "sigma": sg[:mk], "mkept": mk,
                "timing": {f: getattr(t, f) for f, _ in Timing._fields_}}
