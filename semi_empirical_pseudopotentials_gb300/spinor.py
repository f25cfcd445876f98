"""The non-local spin-orbit operator of the spinor filter (the reference's
spinors/filterSpinors/), applied on the GPU by libsep_gb300.so.

Spinors are 2 ngrid complex values: the spin-up grid, then the spin-down
grid.  Neighbour lists are structured arrays with the fields of the
reference's nlc_st (NLC_DTYPE, filterSpinors/fd.h:55-60), natom x nnlc, of
which nl[a] entries are used for atom a; the reference's own nlc arrays have
this layout.

* ``neighbour_lists(vx, vy, vz, rxyz, vso, rnlcut2)``: the lists of
  filterSpinors/init.c:114-181 (host code of the library);
* ``nonlocal_potential(psi, nlc, nl, sigma, dv)``: the Gaussian form,
  filterSpinors/hamiltonian.c:81-190;
* ``nonlocal_potential_kb(psi, nlc, nl, elkb, dv)``: the Kleinman-Bylander
  form, filterSpinors/hamiltonian.c:193-401;
* ``SpinorPath(ctx, nlc, nl, sigma=..., elkb=...)``: the spinor filter
  program on a context's grid and potential -- the spinor Hamiltonian, its
  energy range, the Newton filter with complex coefficients and the whole
  pipeline (filterSpinors/main.c:84-175).
"""
import ctypes as C

import numpy as np

from .binding import Timing, _check, lib

NLC_DTYPE = np.dtype([("jxyz", "<i8"), ("y10", "<c16"), ("y11", "<c16"), ("y1_1", "<c16"),
                      ("Vs0G1", "<f8"), ("Vs0G_2", "<f8"), ("r", "<f8"), ("r2_1", "<f8"),
                      ("r2", "<f8"), ("Vr", "<f8")])


def neighbour_lists(vx, vy, vz, rxyz, vso, rnlcut2, nnlc=None):
    """(nlc natom x nnlc, nl) for atoms at rxyz with spin-orbit strengths vso
    on the grid vx x vy x vz (filterSpinors/init.c:114-181).  nnlc defaults
    to the largest count."""
    vx, vy, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in (vx, vy, vz))
    rxyz = np.ascontiguousarray(rxyz, dtype=np.float64).reshape(-1, 3)
    vso = np.ascontiguousarray(vso, dtype=np.float64).ravel()
    natom = len(rxyz)
    if vso.shape != (natom,):
        raise ValueError("vso has one entry per atom")
    dp = C.POINTER(C.c_double)
    nl = np.zeros(natom, dtype=np.int64)
    L = lib()
    args = (len(vx), len(vy), len(vz), vx.ctypes.data_as(dp), vy.ctypes.data_as(dp),
            vz.ctypes.data_as(dp), natom, rxyz.ctypes.data_as(dp), vso.ctypes.data_as(dp),
            float(rnlcut2))
    lp = C.POINTER(C.c_long)
    if nnlc is None:
        _check(L.sep_spinor_neighbour_lists(*args, 0, None, nl.ctypes.data_as(lp)))
        nnlc = int(nl.max()) if natom else 0
    nlc = np.zeros((natom, int(nnlc)), dtype=NLC_DTYPE)
    _check(L.sep_spinor_neighbour_lists(*args, int(nnlc), nlc.ctypes.data_as(C.c_void_p),
                                        nl.ctypes.data_as(lp)))
    return nlc, nl


def _apply(psi, nlc, nl, sigma, dv, flagkb, elkb):
    psi = np.ascontiguousarray(psi, dtype=np.complex128).ravel()
    if psi.size % 2:
        raise ValueError("a spinor has 2 ngrid values")
    ngrid = psi.size // 2
    nlc = np.ascontiguousarray(nlc, dtype=NLC_DTYPE)
    if nlc.ndim != 2:
        raise ValueError("nlc is natom x nnlc")
    nl = np.ascontiguousarray(nl, dtype=np.int64)
    natom, nnlc = nlc.shape
    if nl.shape != (natom,):
        raise ValueError("nl has one entry per atom")
    out = np.zeros_like(psi)
    dp = C.POINTER(C.c_double)
    el = None
    if flagkb:
        el = np.ascontiguousarray(elkb, dtype=np.float64)
        if el.shape != (2 * natom,):
            raise ValueError("elkb has 2 natom entries")
    _check(lib().sep_spinor_vso(psi.view(np.float64).ctypes.data_as(dp), ngrid, natom, nnlc,
                                nlc.ctypes.data_as(C.c_void_p),
                                nl.ctypes.data_as(C.POINTER(C.c_long)), float(sigma), float(dv),
                                int(flagkb), el.ctypes.data_as(dp) if el is not None else None,
                                out.view(np.float64).ctypes.data_as(dp)))
    return out


def nonlocal_potential(psi, nlc, nl, sigma, dv):
    """Vso psi, Gaussian form (filterSpinors/hamiltonian.c:81-190)."""
    return _apply(psi, nlc, nl, sigma, dv, 0, None)


def nonlocal_potential_kb(psi, nlc, nl, elkb, dv):
    """Vso psi, Kleinman-Bylander form (filterSpinors/hamiltonian.c:193-401)."""
    return _apply(psi, nlc, nl, 1.0, dv, 1, elkb)


class SpinorPath:
    """The spinor filter program on the grid and local potential of a
    binding.Context (FP64).  Spinors are complex arrays of 2 ngrid values."""

    def __init__(self, ctx, nlc, nl, sigma=None, elkb=None):
        self.ctx = ctx
        nlc = np.ascontiguousarray(nlc, dtype=NLC_DTYPE)
        nl = np.ascontiguousarray(nl, dtype=np.int64)
        natom, nnlc = nlc.shape
        flagkb = elkb is not None
        el = None
        if flagkb:
            el = np.ascontiguousarray(elkb, dtype=np.float64)
            if el.shape != (2 * natom,):
                raise ValueError("elkb has 2 natom entries")
        dp = C.POINTER(C.c_double)
        L = lib()
        L.sep_spinor_set_operator.argtypes = [C.c_void_p, C.c_long, C.c_long, C.c_void_p,
                                              C.c_void_p, C.c_double, C.c_int, C.c_void_p]
        _check(L.sep_spinor_set_operator(ctx.h, natom, nnlc, nlc.ctypes.data, nl.ctypes.data,
                                         float(sigma or 0.0), int(flagkb),
                                         el.ctypes.data if el is not None else None))
        self._keep = (nlc, nl, el)
        self.n = ctx.ngrid

    def _spinors(self, psi):
        z = np.ascontiguousarray(psi, dtype=np.complex128)
        return z.reshape(-1, 2 * self.n)

    def hamiltonian(self, psi):
        """H psi (filterSpinors/hamiltonian.c:8-46), one or more spinors."""
        z = self._spinors(psi)
        out = np.empty_like(z)
        L = lib()
        L.sep_spinor_hamiltonian.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]
        _check(L.sep_spinor_hamiltonian(self.ctx.h, z.ctypes.data, out.ctypes.data, z.shape[0]))
        return out.reshape(np.shape(psi))

    def energy_range(self):
        """(vmin, dE, iterations) of filterSpinors/energy.c:49-109."""
        vmin, dE, it = C.c_double(), C.c_double(), C.c_long()
        L = lib()
        L.sep_spinor_energy_range.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _check(L.sep_spinor_energy_range(self.ctx.h, C.byref(vmin), C.byref(dE), C.byref(it)))
        return vmin.value, dE.value, it.value

    def filter(self, start, an, zn, dE_1, vmin):
        """filterSpinors/filter.c:48-80: [ns, ms, 2 ngrid] from [ns, 2 ngrid]
        start spinors and complex coefficients an [ms, nc]."""
        st = self._spinors(start)
        an = np.asarray(an, dtype=np.complex128)
        ar = np.ascontiguousarray(an.real)
        ai = np.ascontiguousarray(an.imag)
        zn = np.ascontiguousarray(zn, dtype=np.float64)
        ms, nc = ar.shape
        out = np.empty((st.shape[0], ms, 2 * self.n), dtype=np.complex128)
        L = lib()
        L.sep_spinor_filter.argtypes = [C.c_void_p, C.c_void_p, C.c_long, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_long, C.c_long, C.c_double,
                                        C.c_double, C.c_void_p]
        _check(L.sep_spinor_filter(self.ctx.h, st.ctypes.data, st.shape[0], ar.ctypes.data,
                                   ai.ctypes.data, zn.ctypes.data, ms, nc, float(dE_1),
                                   float(vmin), out.ctypes.data))
        return out

    def pipeline(self, start, el, nc, vmin=0.0, dE=0.0, want_psi=False):
        """filterSpinors/main.c:84-175 from given start spinors [ns, 2 ngrid]."""
        st = self._spinors(start)
        el = np.ascontiguousarray(el, dtype=np.float64)
        ns, ms = st.shape[0], len(el)
        m = ns * ms
        ev, sg = np.zeros(m), np.zeros(m)
        psi = np.empty((m, 2 * self.n), dtype=np.complex128) if want_psi else None
        k = C.c_long()
        t = Timing()
        L = lib()
        L.sep_spinor_pipeline.argtypes = [C.c_void_p, C.c_void_p, C.c_long, C.c_void_p, C.c_long,
                                          C.c_long, C.c_double, C.c_double, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _check(L.sep_spinor_pipeline(self.ctx.h, st.ctypes.data, ns, el.ctypes.data, ms, int(nc),
                                     float(vmin), float(dE),
                                     psi.ctypes.data if psi is not None else None,
                                     ev.ctypes.data, sg.ctypes.data, C.byref(k), C.byref(t)))
        kk = k.value
        return {"eval": ev[:kk], "sigma": sg[:kk], "mkept": kk,
                "psi": None if psi is None else psi[:kk],
                "timing": {f: getattr(t, f) for f, _ in Timing._fields_}}
