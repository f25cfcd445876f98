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
  form, filterSpinors/hamiltonian.c:193-401.
"""
import ctypes as C

import numpy as np

from .binding import _check, lib

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
