"""The reference's own entry points (include/sep_fd_compat.h), called the way
filter/main.c:64-142 calls them, against the reference program's output
(tests/golden/ref_small.npz: a fixed-seed run of the reference's sources).
Structs travel by value exactly as in the reference (filter/fd.h:23-36)."""
import ctypes as C
import os

import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from semi_empirical_pseudopotentials_gb300 import binding

pytestmark = pytest.mark.gpu


class ParSt(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dx", "dy", "dz", "dr", "dkx", "dky", "dkz", "dv", "dt", "xmin", "xmax", "ymin",
        "ymax", "zmin", "zmax", "Vmin", "Vmax", "dE", "dE_1", "Elmin", "Elmax", "Ekinmax")]


class LongSt(C.Structure):
    _fields_ = [(n, C.c_long) for n in (
        "natom", "lumo", "homo", "ms", "ns", "nc", "npot", "mstot", "nx", "ny", "nz", "ngrid",
        "natomtype", "nthreads")] + [("nx_1", C.c_double), ("ny_1", C.c_double),
                                     ("nz_1", C.c_double)]


def _lib():
    path = os.path.join(os.path.dirname(binding.LIB_PATH), "libsep_fdcompat.so")
    L = C.CDLL(path)
    L.portho.restype = C.c_long
    L.norm.restype = C.c_double
    L.normalize.restype = C.c_double
    L.energy.restype = C.c_double
    return L


def test_reference_main_flow(golden, tmp_path, monkeypatch):
    g = golden("ref_small.npz")
    monkeypatch.chdir(tmp_path)  # filtering() writes the reference's per-cycle files
    L = _lib()
    nx, ny, nz = (int(v) for v in g["dims"])
    N = nx * ny * nz
    ms, ns, nc = 3, 4, 128
    ist = LongSt(ms=ms, ns=ns, nc=nc, mstot=ms * ns, nx=nx, ny=ny, nz=nz, ngrid=N, nthreads=1,
                 natomtype=17, npot=8192, nx_1=1.0 / nx, ny_1=1.0 / ny, nz_1=1.0 / nz)
    par = ParSt(dx=float(g["dx"]), dy=float(g["dy"]), dz=float(g["dz"]), dv=float(g["dv"]),
                Vmin=float(g["vmin"]), Vmax=float(g["vmax"]),
                Ekinmax=10.0 * ((1.0 / ny) * (1.0 / nx) * (1.0 / nz)))  # init.c:137
    potl, ksqr = np.ascontiguousarray(g["potl"]), np.ascontiguousarray(g["ksqr"])
    dp = C.POINTER(C.c_double)
    psi = np.zeros(2 * N)
    phi = np.zeros(2 * N)
    null = C.c_void_p()
    L.get_energy_range(psi.ctypes.data_as(dp), phi.ctypes.data_as(dp), potl.ctypes.data_as(dp),
                       None, None, None, ksqr.ctypes.data_as(dp), C.byref(par), ist, null, null,
                       null)
    assert abs(par.dE - float(g["run_dE"])) <= 1e-9 * float(g["run_dE"])
    par.dt = (nc / (2.5 * par.dE)) ** 2                                  # main.c:70
    an = np.zeros(2 * nc * ms)
    zn = np.zeros(nc)
    el = np.ascontiguousarray(g["el"])
    L.coefficient(an.ctypes.data_as(dp), zn.ctypes.data_as(dp), el.ctypes.data_as(dp), par, ist)
    ar, ai, zref = sep.coefficients(el, nc, par.dE, par.Vmin, par.dt)
    assert np.array_equal(an[0::2].reshape(ms, nc), ar) and np.array_equal(zn, zref)
    # start states: one seed, consecutive draws (main.c:82-89)
    start = sep.start_states(int(g["run_seed"]), ns, N, par.dv)
    psitot = np.zeros(ms * ns * N)
    for s in range(ns):
        for e in range(ms):
            psitot[(s * ms + e) * N:(s * ms + e + 1) * N] = start[s]
    idum = C.c_long(0)
    for s in range(ns):                                                  # main.c:94-98
        blk = psitot[s * ms * N:].ctypes.data_as(dp)
        L.filtering(blk, potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp),
                    an.ctypes.data_as(dp), zn.ctypes.data_as(dp), el.ctypes.data_as(dp), ist,
                    par, C.c_long(0), C.c_long(s), C.byref(idum))
    # the per-cycle files of filter/filter.c:37-47: the filtered block as raw
    # doubles, and "%ld %.16g %.16g" lines of (index, E, target)
    assert np.array_equal(np.fromfile(tmp_path / "psi-filt-0-3.dat"),
                          psitot[3 * ms * N:4 * ms * N])
    rows = np.loadtxt(tmp_path / "eval-filt-0-3.dat", ndmin=2)
    assert np.array_equal(rows[:, 0], np.arange(ms))
    assert np.allclose(rows[:, 2], el, rtol=1e-15, atol=0)
    ist.mstot = L.portho(psitot.ctypes.data_as(dp), C.c_double(par.dv), ist)   # main.c:110
    assert ist.mstot == len(g["run_eval"])
    L.normalize_all(psitot.ctypes.data_as(dp), C.c_double(par.dv), C.c_long(ist.mstot),
                    C.c_long(N), C.c_long(1))
    ev = np.zeros(ist.mstot)
    L.Hmatreal(psi.ctypes.data_as(dp), phi.ctypes.data_as(dp), psitot.ctypes.data_as(dp),
               potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp), ev.ctypes.data_as(dp), ist, par,
               null, null, null)
    L.normalize_all(psitot.ctypes.data_as(dp), C.c_double(par.dv), C.c_long(ist.mstot),
                    C.c_long(N), C.c_long(1))
    sg = np.zeros(ist.mstot)
    L.calc_sigma_E(psi.ctypes.data_as(dp), phi.ctypes.data_as(dp), psitot.ctypes.data_as(dp),
                   potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp), sg.ctypes.data_as(dp), ist,
                   par, null, null, null)
    assert np.allclose(ev, g["run_eval"], rtol=0, atol=1e-8)
    assert np.allclose(sg, g["run_sigma"], rtol=2e-5, atol=1e-7)


def test_hamiltonian_and_hnorm_entry_points(golden):
    g = golden("ref_small.npz")
    L = _lib()
    nx, ny, nz = (int(v) for v in g["dims"])
    N = nx * ny * nz
    ist = LongSt(nx=nx, ny=ny, nz=nz, ngrid=N, ms=3, nc=128, nthreads=1)
    par = ParSt(dx=float(g["dx"]), dy=float(g["dy"]), dz=float(g["dz"]), dv=float(g["dv"]),
                Vmin=float(g["vmin"]), Ekinmax=10.0 * ((1.0 / ny) * (1.0 / nx) * (1.0 / nz)),
                dE=float(g["dE"]), dE_1=4.0 / float(g["dE"]))
    dp = C.POINTER(C.c_double)
    potl, ksqr = np.ascontiguousarray(g["potl"]), np.ascontiguousarray(g["ksqr"])
    null = C.c_void_p()
    phi = np.ascontiguousarray(g["h_in"]).copy()
    tmp = np.zeros_like(phi)
    L.hamiltonian(phi.ctypes.data_as(dp), tmp.ctypes.data_as(dp), potl.ctypes.data_as(dp),
                  ksqr.ctypes.data_as(dp), ist, par, null, null, null)
    ref = g["h_out"]
    assert np.abs(phi - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.array_equal(tmp, g["h_in"])  # psi <- the old phi, as hamiltonian.c:14
    psim1 = np.ascontiguousarray(g["h_in"]).copy()
    psin = psim1.copy()
    L.hnorm(psim1.ctypes.data_as(dp), psin.ctypes.data_as(dp), potl.ctypes.data_as(dp),
            ksqr.ctypes.data_as(dp), par, C.c_double(0.37), ist, null, null, null)
    assert np.abs(psin - g["hnorm_out"]).max() <= 1e-12 * np.abs(g["hnorm_out"]).max()
