"""Generate the golden fixtures under tests/golden/ (run where the reference
checkout exists; the outputs are committed, the GPU machine never needs the
reference).

Fixtures:
* in13_p16.npz  -- the reference's own end-to-end fixture
  (filterStrainCube/test/In13_P16): its inputs (atoms, per-atom strain scale
  from strain.dat, the In/P potential tables, input.par values) and its
  published outputs (eval.dat Ritz values and sigmas; run.dat's Vmin, Vmax,
  dT, dE, dt and ortho cutoff).  Data copied as-is.
* zb_cdse_formfactor.npz -- pseudopotFitting/TESTS/zb_cdse: CdParams.par,
  SeParams.par, volPerAtom (run.dat) and the pot_Cd_0.dat / pot_Se_0.dat
  real-space tables that pot.c wrote from them (printed with %g).
* ref_small.npz -- outputs of the reference's own filter sources, compiled
  here by oracle/Makefile.ref, on a small synthetic nanocrystal with a
  non-cubic grid: ran_nrc sequences, init_psi states, init()'s potl / ksqr /
  Vmin, coefficient(), hamiltonian(), hnorm(), filter(), energy_all(),
  get_energy_range(), and a full fixed-seed filter_ref run (eval.dat).

* config0_ref.npz -- the reference's own filter program on the benchmark's
  smallest configuration (CONFIG0) with a fixed start seed: eval.dat and the
  run's dE, Vmin, dt.

usage: python tests/golden/make_golden.py [/path/to/reference] [--config0]
  (--config0: only config0_ref.npz)
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from semi_empirical_pseudopotentials_gb300 import systems  # noqa: E402

_ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
REF = build_oracle.reference_dir(_ARGS[0] if _ARGS else None)


# ---- filter/fd.h:23-36 struct layouts --------------------------------------
class ParSt(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dx", "dy", "dz", "dr", "dkx", "dky", "dkz", "dv", "dt", "xmin", "xmax", "ymin",
        "ymax", "zmin", "zmax", "Vmin", "Vmax", "dE", "dE_1", "Elmin", "Elmax", "Ekinmax")]


class LongSt(C.Structure):
    _fields_ = [(n, C.c_long) for n in (
        "natom", "lumo", "homo", "ms", "ns", "nc", "npot", "mstot", "nx", "ny", "nz", "ngrid",
        "natomtype", "nthreads")] + [("nx_1", C.c_double), ("ny_1", C.c_double),
                                     ("nz_1", C.c_double)]


class AtmSt(C.Structure):
    _fields_ = [("natyp", C.c_long), ("atyp", C.c_char * 3)]


def fixture_in13():
    d = os.path.join(REF, "filterStrainCube/test/In13_P16")
    inp = open(os.path.join(d, "input.par")).read().split()
    nx, ny, nz, ms, ns, nc = (int(v) for v in inp[:6])
    elmin, elmax, nthreads = float(inp[6]), float(inp[7]), int(inp[8])
    lines = open(os.path.join(d, "conf.par")).read().split("\n")
    natom = int(lines[0])
    sym, xyz = [], []
    for ln in lines[1:1 + natom]:
        p = ln.split()
        sym.append(p[0])
        xyz.append([float(v) for v in p[1:4]])
    strain = np.loadtxt(os.path.join(d, "strain.dat"), usecols=(6,))
    # reference type ids (filter/read.c:126-152)
    type_id = {"Cd": 0, "In": 2, "P1": 8, "P2": 9, "P": 16}
    # unshifted tables [17, 1024] by type id; files for In and P, and the
    # Gaussian a exp(-r^2/b) of filterStrainCube/read.c:52-56,111-118 for the
    # P1/P2 ligands on the r grid of potCd.par (type 0)
    tab_r = np.zeros((17, 1024))
    tab_v = np.zeros((17, 1024))
    tab_n = np.zeros(17, dtype=np.int64)
    for s in ("Cd", "In", "P"):
        t = np.loadtxt(os.path.join(d, f"pot{s}.par"))
        tab_r[type_id[s], :len(t)] = t[:, 0]
        tab_v[type_id[s], :len(t)] = t[:, 1]
        tab_n[type_id[s]] = len(t)
    libm = C.CDLL("libm.so.6")
    libm.exp.restype = C.c_double
    libm.exp.argtypes = [C.c_double]
    for s, a in (("P1", 0.64), ("P2", -0.384)):
        j = type_id[s]
        tab_n[j] = tab_n[0]
        for i in range(tab_n[0]):
            r = tab_r[0, i]
            tab_r[j, i] = r
            tab_v[j, i] = a * libm.exp(-(r * r) / 2.2287033)
    ev = np.loadtxt(os.path.join(d, "eval.dat"))
    np.savez_compressed(
        os.path.join(HERE, "in13_p16.npz"), dims=np.array([nx, ny, nz]),
        ms=ms, ns=ns, nc=nc, elmin=elmin, elmax=elmax,
        types=np.array([type_id[s] for s in sym]), xyz_raw=np.array(xyz), strain_scale=strain,
        tab_r=tab_r, tab_v=tab_v, tab_n=tab_n, eval=ev[:, 1], sigma=ev[:, 2],
        # filterStrainCube/test/In13_P16/run.dat:46-57
        vmin=-1.44656, vmax=1.35926, dT=24.4726, dE=13.3627, dt=939.57, cutoff=158)


def fixture_zb_cdse():
    d = os.path.join(REF, "pseudopotFitting/TESTS/zb_cdse")
    cd = np.loadtxt(os.path.join(d, "CdParams.par"))
    se = np.loadtxt(os.path.join(d, "SeParams.par"))
    np.savez_compressed(
        os.path.join(HERE, "zb_cdse_formfactor.npz"), cd_params=cd, se_params=se,
        vol_per_atom=187.56808402,  # TESTS/zb_cdse/run.dat:4
        pot_cd=np.loadtxt(os.path.join(d, "pot_Cd_0.dat")),
        pot_se=np.loadtxt(os.path.join(d, "pot_Se_0.dat")))


def small_reference_outputs():
    refdir = build_oracle.build_ref(REF)
    L = C.CDLL(os.path.join(refdir, "libsepref.so"))
    L.ran_nrc.restype = C.c_double
    L.fftw_plan_dft_3d.restype = C.c_void_p
    L.fftw_plan_dft_3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_uint]
    L.fftw_malloc.restype = C.c_void_p
    dp = C.POINTER(C.c_double)

    def p(a):
        return a.ctypes.data_as(dp)

    out = {}
    for seed in (-874917403, -12345, -1131359211):
        idum = C.c_long(seed)
        out[f"ran_{-seed}"] = np.array([L.ran_nrc(C.byref(idum)) for _ in range(300)])

    # small synthetic system on a non-cubic grid
    S = systems.make_system("small", 0.6, (16, 18, 20), ms=3, ns=4, nc=128, seed=7,
                            elmin=-0.5, elmax=0.5)
    tabs = {t: _form_factor_table(a, S.vol_per_atom) for t, a in S.params.items()}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        systems.write_reference_inputs(S, tmp, nthreads=1, tables=tabs)
        os.chdir(tmp)
        try:
            par, ist = ParSt(), LongSt()
            argv = (C.c_char_p * 1)(b"x")
            L.init_size(C.c_long(1), argv, C.byref(par), C.byref(ist))
            N = ist.ngrid
            potl, ksqr = np.zeros(N), np.zeros(N)
            vx, vy, vz = np.zeros(ist.nx), np.zeros(ist.ny), np.zeros(ist.nz)
            rx, ry, rz = np.zeros(ist.natom), np.zeros(ist.natom), np.zeros(ist.natom)
            atm = (AtmSt * ist.natom)()
            el = np.zeros(ist.ms)
            scratch = L.fftw_malloc(C.c_size_t(16 * N))
            pf, pb = C.c_void_p(), C.c_void_p()
            L.init(p(potl), p(vx), p(vy), p(vz), p(ksqr), p(rx), p(ry), p(rz), atm, C.byref(par),
                   p(el), C.byref(ist), C.byref(pf), C.byref(pb), C.c_void_p(scratch))
            pf = L.fftw_plan_dft_3d(ist.nz, ist.ny, ist.nx, scratch, scratch, -1, 0)
            pb = L.fftw_plan_dft_3d(ist.nz, ist.ny, ist.nx, scratch, scratch, 1, 0)
            pf, pb = C.c_void_p(pf), C.c_void_p(pb)
            out.update(dims=np.array([ist.nx, ist.ny, ist.nz]), potl=potl.copy(),
                       ksqr=ksqr.copy(), vx=vx.copy(), vy=vy.copy(), vz=vz.copy(),
                       rx=rx.copy(), ry=ry.copy(), rz=rz.copy(), el=el.copy(), vmin=par.Vmin,
                       vmax=par.Vmax, dv=par.dv, dx=par.dx, dy=par.dy, dz=par.dz,
                       xmin=par.xmin, ymin=par.ymin, zmin=par.zmin,
                       types=np.array([a.natyp for a in atm]),
                       tab_r=np.stack([tabs[0][0], tabs[1][0]]),
                       tab_v=np.stack([tabs[0][1], tabs[1][1]]),
                       params=np.stack([S.params[0], S.params[1]]), vol_per_atom=S.vol_per_atom)
            # init_psi (filter/init.c:236-251) with nthreads = 1 sums in order
            idum = C.c_long(-777)
            psi = np.zeros(N, dtype=np.complex128)
            starts = []
            for _ in range(2):
                L.init_psi(psi.ctypes.data_as(dp), ist, par, C.byref(idum))
                starts.append(psi.real.copy())
            out["init_psi_seed777"] = np.stack(starts)
            # hamiltonian on a random complex state (filter/hamiltonian.c:11-23)
            rng = np.random.default_rng(3)
            z = rng.standard_normal(N) + 1j * rng.standard_normal(N)
            phi = z.copy()
            tmpz = np.zeros(N, dtype=np.complex128)
            L.hamiltonian(phi.ctypes.data_as(dp), tmpz.ctypes.data_as(dp), p(potl), p(ksqr), ist,
                          par, pf, pb, C.c_void_p(scratch))
            out["h_in"], out["h_out"] = z, phi.copy()
            # energy range (filter/energy.c:53-83)
            par2 = ParSt.from_buffer_copy(par)
            a = np.zeros(N, dtype=np.complex128)
            b = np.zeros(N, dtype=np.complex128)
            L.get_energy_range(a.ctypes.data_as(dp), b.ctypes.data_as(dp), p(potl), p(vx), p(vy),
                               p(vz), p(ksqr), C.byref(par2), ist, pf, pb, C.c_void_p(scratch))
            out["dE"] = par2.dE
            # coefficients (filter/coeff.c:16-63) at nc = 128 and nc = 1024
            for nc in (128, 1024):
                ist2 = LongSt.from_buffer_copy(ist)
                ist2.nc = nc
                par3 = ParSt.from_buffer_copy(par2)
                par3.dt = (nc / (2.5 * par3.dE)) ** 2
                an = np.zeros(nc * ist.ms, dtype=np.complex128)
                zn = np.zeros(nc)
                L.coefficient(an.ctypes.data_as(dp), p(zn), p(el), par3, ist2)
                out[f"an_{nc}"] = an.reshape(ist.ms, nc)
                out[f"zn_{nc}"] = zn
                out[f"dt_{nc}"] = par3.dt
            # hnorm (filter/hnorm.c:11-25)
            psim1 = z.copy()
            psin = z.copy()
            L.hnorm(psim1.ctypes.data_as(dp), psin.ctypes.data_as(dp), p(potl), p(ksqr), par2,
                    C.c_double(0.37), ist, pf, pb, C.c_void_p(scratch))
            out["hnorm_out"] = psin.copy()
            # one filter cycle (filter/filter.c:59-83) at nc = 128
            ist2 = LongSt.from_buffer_copy(ist)
            ist2.nc = 128
            par3 = ParSt.from_buffer_copy(par2)
            par3.dt = out["dt_128"]
            an = out["an_128"].copy()
            zn = out["zn_128"].copy()
            psin = np.zeros(N, dtype=np.complex128)
            psin.real = starts[0]
            psim1 = np.zeros(N, dtype=np.complex128)
            psi0 = np.zeros(ist.ms * N)
            L.filter(psin.ctypes.data_as(dp), psim1.ctypes.data_as(dp), p(psi0), p(potl),
                     p(ksqr), par3, an.ctypes.data_as(dp), p(zn), ist2, pf, pb,
                     C.c_void_p(scratch), C.c_long(0), C.c_long(0))
            out["filter_out"] = psi0.reshape(ist.ms, N).copy()
            # energy_all (filter/energy.c:28-49) of the normalised filter output
            L.normalize_all(p(psi0), C.c_double(par.dv), C.c_long(ist.ms), C.c_long(N),
                            C.c_long(1))
            ene = np.zeros(ist.ms)
            L.energy_all(a.ctypes.data_as(dp), b.ctypes.data_as(dp), p(psi0), p(potl), p(ksqr),
                         p(ene), ist, par2, pf, pb, C.c_void_p(scratch))
            out["filter_norm"] = psi0.reshape(ist.ms, N).copy()
            out["energy_all"] = ene
        finally:
            os.chdir(cwd)
        # full fixed-seed run of the reference program (nthreads = 1)
        res = subprocess.run([os.path.join(refdir, "filter_ref"), "-24680", "1"], cwd=tmp,
                             capture_output=True, text=True, check=True)
        ev = np.loadtxt(os.path.join(tmp, "eval.dat"))
        out["run_seed"] = -24680
        out["run_eval"] = ev[:, 1]
        out["run_sigma"] = ev[:, 2]
        for ln in res.stdout.splitlines():
            if ln.startswith("nc = "):
                f = ln.split()
                out["run_dt"] = float(f[5])
                out["run_dE"] = float(f[8])
                out["run_vmin"] = float(f[11])
    np.savez_compressed(os.path.join(HERE, "ref_small.npz"), **out)


# The benchmark's smallest configuration: the 1.2 nm sphere (275 atoms) with
# the seeded a0 = +-10 form factors on its 64^3 grid, 8 start states x 4
# targets, nc = 1024, FP64.  The targets cover [-3.25, -2.95] Ha, the window
# of the 128^3 benchmark workload.
CONFIG0 = dict(radius_nm=1.2, n=64, ms=4, ns=8, nc=1024, seed=0, elmin=-3.25, elmax=-2.95,
               start_seed=-271828)


def config0_reference_run(nthreads=8):
    """config0_ref.npz: the reference's own filter program (filter_ref, built by
    oracle/Makefile.ref from filter/*.c) on CONFIG0 with a fixed start seed:
    eval.dat (Ritz values, sigma), the kept count and its dE, Vmin, dt."""
    refdir = build_oracle.build_ref(REF)
    c = CONFIG0
    S = systems.make_system("config0", c["radius_nm"], c["n"], c["ms"], c["ns"], c["nc"],
                            seed=c["seed"], elmin=c["elmin"], elmax=c["elmax"])
    tabs = {t: _form_factor_table(a, S.vol_per_atom) for t, a in S.params.items()}
    with tempfile.TemporaryDirectory() as tmp:
        systems.write_reference_inputs(S, tmp, nthreads=nthreads, tables=tabs)
        res = subprocess.run([os.path.join(refdir, "filter_ref"), str(c["start_seed"]),
                              str(nthreads)], cwd=tmp, capture_output=True, text=True,
                             check=True)
        ev = np.loadtxt(os.path.join(tmp, "eval.dat"))
    out = dict(CONFIG0)
    out.update(eval=ev[:, 1], sigma=ev[:, 2], mkept=len(ev))
    for ln in res.stdout.splitlines():
        if ln.startswith("nc = "):
            f = ln.split()
            out.update(dt=float(f[5]), dE=float(f[8]), vmin=float(f[11]))
    np.savez_compressed(os.path.join(HERE, "config0_ref.npz"), **out)


def _form_factor_table(a, vol):
    from oracle import oracle as O

    return O.form_factor_table(a, vol)


if __name__ == "__main__":
    if "--config0" not in sys.argv:
        fixture_in13()
        fixture_zb_cdse()
        small_reference_outputs()
    config0_reference_run()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
