"""Golden vectors for the spin-orbit operator of the spinor filter
(spinors/filterSpinors/), from the reference's own code.

Run in a container that has the reference checkout (not on a GPU machine), after
`python oracle/build_oracle.py` has compiled oracle/_ref/libspinorref.so from
the reference's sources:

    python tests/golden/make_spinor_fixture.py

On a 16 x 16 x 14 grid (0.6 bohr) with three atoms it calls the
reference's init_list (filterSpinors/init.c:114-181) for the neighbour
lists, fills the Kleinman-Bylander fields (Vs0G1, Vs0G_2, Elkb; made by
init_kb in a full run) with seeded values, and applies nonlocal_potential
(Gaussian form, hamiltonian.c:81-190) and nonlocal_potential_kb
(hamiltonian.c:193-401) to a seeded random spinor.  It then applies the
whole spinor hamiltonian() (hamiltonian.c:8-46) in both forms and runs a
6-step Newton filter() (filter.c:48-80) with complex coefficients for two
targets, with a local potential of Gaussian wells at the atoms.  The arrays
go to tests/golden/spinor_vso.npz.
"""
import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "..", "oracle", "_ref", "libspinorref.so")


class LongSt(C.Structure):   # filterSpinors/fd.h:31-40
    _fields_ = [(n, C.c_long) for n in (
        "natom", "lumo", "homo", "flaghomo", "nsemicond", "ms", "ns", "nc", "npot", "mstot",
        "mstotngrid", "nspinngrid", "nx", "ny", "nz", "ngrid", "nspin", "nnlc", "natomtype",
        "nthreads", "flagkb")] + [("nx_1", C.c_double), ("ny_1", C.c_double),
                                  ("nz_1", C.c_double)]


class ParSt(C.Structure):    # filterSpinors/fd.h:24-29
    _fields_ = [(n, C.c_double) for n in (
        "dx", "dy", "dz", "dr", "dkx", "dky", "dkz", "dv", "dt", "xmin", "xmax", "ymin", "ymax",
        "zmin", "zmax", "Vmin", "Vmax", "dE", "dE_1", "Elmin", "Elmax", "Ekinmax", "Rnlcut2",
        "sigma", "sigma_1")]


class AtmSt(C.Structure):    # filterSpinors/fd.h:46-50
    _fields_ = [("natyp", C.c_long), ("atyp", C.c_char * 3), ("Vso", C.c_double),
                ("initE", C.c_double)]


def main():
    from oracle.spinor_oracle import NLC_DTYPE

    L = C.CDLL(os.path.abspath(LIB))
    nx, ny, nz, h = 16, 16, 14, 0.6
    ngrid = nx * ny * nz
    vx = -0.5 * nx * h + h * np.arange(nx)
    vy = -0.5 * ny * h + h * np.arange(ny)
    vz = -0.5 * nz * h + h * np.arange(nz)
    rxyz = np.array([[0.31, -0.42, 0.17], [-1.93, 1.12, -0.86], [1.71, 1.29, 1.03]])
    vso = np.array([0.0813, -0.0457, 0.1221])
    nat = len(rxyz)
    rnlcut2 = 0.49 * 6.0 * np.log(10.0)              # init.c:99
    nnlc = 600                                      # > the ~340 points per atom
    ist = LongSt(natom=nat, nsemicond=nat, nx=nx, ny=ny, nz=nz, ngrid=ngrid, nspin=2,
                 nspinngrid=2 * ngrid, nnlc=nnlc, nthreads=1)
    par = ParSt(dx=h, dy=h, dz=h, dv=h ** 3, Rnlcut2=rnlcut2, sigma=h,
                sigma_1=np.sqrt(0.5) / h)            # init.c:96-97
    atm = (AtmSt * nat)()
    for a in range(nat):
        atm[a].Vso = vso[a]
    nlc = np.zeros(nat * nnlc, dtype=NLC_DTYPE)
    nl = np.zeros(nat, dtype=np.int64)
    dp = C.POINTER(C.c_double)
    rx, ry, rz = (np.ascontiguousarray(rxyz[:, k]) for k in range(3))
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:      # init_list writes list.dat
        os.chdir(tmp)
        try:
            L.init_list(nlc.ctypes.data_as(C.c_void_p), nl.ctypes.data_as(C.c_void_p),
                        vx.ctypes.data_as(dp), vy.ctypes.data_as(dp), vz.ctypes.data_as(dp),
                        rx.ctypes.data_as(dp), ry.ctypes.data_as(dp), rz.ctypes.data_as(dp),
                        atm, par, ist)
        finally:
            os.chdir(cwd)
    rng = np.random.default_rng(2026)
    nlc["Vs0G1"] = rng.normal(size=nlc.shape)
    nlc["Vs0G_2"] = rng.normal(size=nlc.shape)
    elkb = rng.uniform(0.5, 2.0, size=2 * nat)
    psi = rng.normal(size=2 * ngrid) + 1j * rng.normal(size=2 * ngrid)
    out_g = np.zeros(2 * ngrid, dtype=np.complex128)
    out_k = np.zeros(2 * ngrid, dtype=np.complex128)
    L.nonlocal_potential(out_g.ctypes.data_as(C.c_void_p), psi.ctypes.data_as(C.c_void_p), ist,
                         par, nlc.ctypes.data_as(C.c_void_p), nl.ctypes.data_as(C.c_void_p))
    L.nonlocal_potential_kb(out_k.ctypes.data_as(C.c_void_p), psi.ctypes.data_as(C.c_void_p),
                            ist, par, nlc.ctypes.data_as(C.c_void_p),
                            nl.ctypes.data_as(C.c_void_p), elkb.ctypes.data_as(dp))
    # the whole spinor Hamiltonian (filterSpinors/hamiltonian.c:8-46) in both
    # spin-orbit forms, and a short Newton filter (filter.c:48-80), through
    # the reference's own routines with FFT plans of the oracle's shim
    import semi_empirical_pseudopotentials_gb300 as sep

    ksqr = sep.ksqr((nx, ny, nz), (h, h, h), ekinmax=20.0)   # init.c:23, 442-460
    zz, yy, xx = np.meshgrid(vz, vy, vx, indexing="ij")
    potl = np.zeros(ngrid)
    for a in range(nat):
        d2 = (xx - rxyz[a, 0]) ** 2 + (yy - rxyz[a, 1]) ** 2 + (zz - rxyz[a, 2]) ** 2
        potl -= 0.4 * np.exp(-0.5 * d2).ravel()
    L.fftw_malloc.restype = C.c_void_p
    L.fftw_plan_dft_3d.restype = C.c_void_p
    buf = C.c_void_p(L.fftw_malloc(C.c_size_t(16 * ngrid)))
    planfw = C.c_void_p(L.fftw_plan_dft_3d(nz, ny, nx, buf, buf, -1, 0))
    planbw = C.c_void_p(L.fftw_plan_dft_3d(nz, ny, nx, buf, buf, 1, 0))
    vp = C.c_void_p
    hpsi = {}
    for flag, name in ((0, "gauss"), (1, "kb")):
        ist.flagkb = flag
        phi = psi.copy()
        scratch = np.zeros_like(psi)
        L.hamiltonian(phi.ctypes.data_as(vp), scratch.ctypes.data_as(vp), potl.ctypes.data_as(dp),
                      ksqr.ctypes.data_as(dp), ist, par, nlc.ctypes.data_as(vp),
                      nl.ctypes.data_as(vp), elkb.ctypes.data_as(dp), planfw, planbw, buf)
        hpsi[name] = phi
    ms, nc = 2, 6
    an = rng.normal(size=ms * nc) + 1j * rng.normal(size=ms * nc)
    zn = rng.uniform(-2.0, 2.0, size=nc)
    par.dE_1, par.Vmin = 4.0 / 3.5, -0.45
    filt_dE_1, filt_vmin = par.dE_1, par.Vmin        # the pipeline run below resets par
    ist.flagkb, ist.ms, ist.nc = 0, ms, nc
    psin = psi.copy()
    psim1 = np.zeros_like(psi)
    psims = np.zeros(ms * 2 * ngrid, dtype=np.complex128)
    with tempfile.TemporaryDirectory() as tmp:      # filter writes prop<tid>.dat
        os.chdir(tmp)
        try:
            L.filter(psin.ctypes.data_as(vp), psim1.ctypes.data_as(vp), psims.ctypes.data_as(vp),
                     potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp), par, nlc.ctypes.data_as(vp),
                     nl.ctypes.data_as(vp), elkb.ctypes.data_as(dp), an.ctypes.data_as(vp),
                     zn.ctypes.data_as(dp), ist, planfw, planbw, buf, C.c_long(0), C.c_long(0))
        finally:
            os.chdir(cwd)
    # Vso psi is zero away from the atoms: kept where it is not; the other
    # outputs as 1024 seeded samples plus the sum and the sum of squares
    outputs = {}
    for name, arr in (("vso_gauss", out_g), ("vso_kb", out_k)):
        nz_idx = np.flatnonzero(arr)
        outputs[name + "_idx"], outputs[name + "_val"] = nz_idx, arr[nz_idx]
    pick = np.sort(np.random.default_rng(99).choice(2 * ngrid, 1024, replace=False))
    for name, arr in (("h_gauss", hpsi["gauss"]), ("h_kb", hpsi["kb"]),
                      ("filter_out", psims.reshape(ms, 2 * ngrid))):
        flat = arr.reshape(-1, 2 * ngrid)
        outputs[name + "_sample"] = flat[:, pick]
        outputs[name + "_sum"] = flat.sum(axis=1)
        outputs[name + "_sumsq"] = (np.abs(flat) ** 2).sum(axis=1)
    outputs["sample_idx"] = pick
    # the reference's whole spinor program on this system (main.c:92-131 with
    # its energy range, coefficients, start states, filtering, portho, Hmat
    # and calc_sigma_E), with a fixed start seed in place of -random()
    ist.flagkb, ist.ms, ist.ns, ist.nc = 0, 2, 2, 64
    ist.mstot = ist.ms * ist.ns
    scratch_a = np.zeros(2 * ngrid, dtype=np.complex128)
    scratch_b = np.zeros(2 * ngrid, dtype=np.complex128)
    el = np.array([-0.36, -0.28])
    with tempfile.TemporaryDirectory() as tmp:       # the stages write log files
        os.chdir(tmp)
        try:
            L.get_energy_range(scratch_a.ctypes.data_as(vp), scratch_b.ctypes.data_as(vp),
                               potl.ctypes.data_as(dp), vx.ctypes.data_as(dp),
                               vy.ctypes.data_as(dp), vz.ctypes.data_as(dp),
                               ksqr.ctypes.data_as(dp), ist, C.byref(par),
                               nlc.ctypes.data_as(vp), nl.ctypes.data_as(vp),
                               elkb.ctypes.data_as(dp), planfw, planbw, buf)
            par.dt = (ist.nc / (2.5 * par.dE)) ** 2          # main.c:84
            an_p = np.zeros(ist.nc * ist.ms, dtype=np.complex128)
            zn_p = np.zeros(ist.nc)
            L.coefficient(an_p.ctypes.data_as(vp), zn_p.ctypes.data_as(dp), el.ctypes.data_as(dp),
                          par, ist)
            seed = -20261203
            idum = C.c_long(seed)
            psitot = np.zeros(ist.mstot * 2 * ngrid, dtype=np.complex128)
            start = np.zeros(2 * ngrid, dtype=np.complex128)
            for jns in range(ist.ns):
                for ispn in range(2):
                    L.init_psi(C.c_void_p(start.ctypes.data + 16 * ispn * ngrid), ist, par,
                               C.byref(idum))
                for jms in range(ist.ms):
                    o = (jns * ist.ms + jms) * 2 * ngrid
                    psitot[o:o + 2 * ngrid] = start
            for jns in range(ist.ns):
                L.filtering(C.c_void_p(psitot.ctypes.data + 16 * jns * ist.ms * 2 * ngrid),
                            potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp),
                            an_p.ctypes.data_as(vp), zn_p.ctypes.data_as(dp),
                            el.ctypes.data_as(dp), ist, par, nlc.ctypes.data_as(vp),
                            nl.ctypes.data_as(vp), elkb.ctypes.data_as(dp), C.c_long(0),
                            C.c_long(jns))
            L.portho.restype = C.c_long
            ist.mstot = L.portho(psitot.ctypes.data_as(vp), C.c_double(par.dv), ist)
            L.normalize_all(psitot.ctypes.data_as(vp), C.c_double(par.dv), C.c_long(ist.mstot),
                            C.c_long(2 * ngrid), C.c_long(1))
            evals = np.zeros(ist.mstot)
            L.Hmat(scratch_a.ctypes.data_as(vp), scratch_b.ctypes.data_as(vp),
                   psitot.ctypes.data_as(vp), potl.ctypes.data_as(dp), ksqr.ctypes.data_as(dp),
                   evals.ctypes.data_as(dp), ist, par, nlc.ctypes.data_as(vp),
                   nl.ctypes.data_as(vp), elkb.ctypes.data_as(dp), planfw, planbw, buf)
            L.normalize_all(psitot.ctypes.data_as(vp), C.c_double(par.dv), C.c_long(ist.mstot),
                            C.c_long(2 * ngrid), C.c_long(1))
            sige = np.zeros(ist.mstot)
            L.calc_sigma_E(scratch_a.ctypes.data_as(vp), scratch_b.ctypes.data_as(vp),
                           psitot.ctypes.data_as(vp), potl.ctypes.data_as(dp),
                           ksqr.ctypes.data_as(dp), sige.ctypes.data_as(dp), ist, par,
                           nlc.ctypes.data_as(vp), nl.ctypes.data_as(vp),
                           elkb.ctypes.data_as(dp), planfw, planbw, buf)
        finally:
            os.chdir(cwd)
    outputs["run_seed"], outputs["run_el"], outputs["run_nc"] = seed, el, ist.nc
    outputs["run_ns"], outputs["run_ms"] = ist.ns, ist.ms
    outputs["run_vmin"], outputs["run_dE"] = par.Vmin, par.dE
    outputs["run_an"], outputs["run_zn"] = an_p.reshape(ist.ms, ist.nc), zn_p
    outputs["run_eval"], outputs["run_sigma"], outputs["run_mkept"] = evals, sige, ist.mstot
    print("energy range", par.Vmin, par.dE, "eval", evals, "sigma", sige)
    width = int(nl.max())                            # entries past nl[a] are unused
    keep = nlc.reshape(nat, nnlc)[:, :width].copy()
    np.savez_compressed(os.path.join(HERE, "spinor_vso.npz"), dims=np.array([nx, ny, nz]), h=h,
                        vx=vx, vy=vy, vz=vz, rxyz=rxyz, vso=vso, rnlcut2=rnlcut2, nnlc=width,
                        nlc=keep.view(np.uint8).reshape(nat, width, NLC_DTYPE.itemsize), nl=nl,
                        elkb=elkb, psi=psi, ksqr=ksqr, potl=potl, an=an.reshape(ms, nc), zn=zn,
                        dE_1=filt_dE_1, vmin=filt_vmin, **outputs)
    print("nl", nl, "|gauss|", np.abs(out_g).max(), "|kb|", np.abs(out_k).max(),
          "|H psi|", np.abs(hpsi["gauss"]).max(), "|filter|", np.abs(psims).max())


if __name__ == "__main__":
    import sys

    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    main()
