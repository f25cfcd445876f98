"""Generate tests/golden/adjoint_ref_fd.npz: the reference-derived gradient of
band-edge eigenvalues with respect to the form-factor parameters.

The reference has no gradients, so the gradient comes from central finite
differences (h = 1e-5) of the reference's own filter program, compiled from its
unmodified sources by oracle/Makefile.ref (oracle/_ref/filter_ref, fixed seed).
Each parameter set is written as the reference's inputs (conf.par, input.par,
potCd.par / potSe.par tables of pseudopotFitting/pot.c:35-63) and the program
is run once per energy window; eval.dat gives the Ritz values.

System: the 0.6 nm zincblende CdSe-like sphere (29 atoms) on a 32^3 grid; the
fitted CdSe form factors of pseudopotFitting/TESTS/zb_cdse (from
zb_cdse_formfactor.npz); 16 start states from seed -314159, nc = 8192,
two windows of two targets each (filter/init.c:210-211):
  valence top   [-0.233, -0.229] Ha  -> the 3 highest converged states (HOMO triplet)
  conduction    [-0.091, -0.050] Ha  -> the 4 lowest converged states (1S_e + 1P_e)

usage: python tests/golden/make_adjoint_fixture.py [/path/to/reference]   (about 25 min)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from oracle import oracle as O  # noqa: E402
from semi_empirical_pseudopotentials_gb300 import systems  # noqa: E402

REF = build_oracle.reference_dir(sys.argv[1] if len(sys.argv) > 1 else None)
RADIUS_NM, N, NS, NC, SEED = 0.6, 32, 16, 8192, -314159
WINDOWS = {"vb": (-0.233, -0.229), "cb": (-0.091, -0.050)}
N_VB, N_CB = 3, 4
H = 1e-5
SIGMA_MAX = 1e-6


def theta0():
    g = np.load(os.path.join(HERE, "zb_cdse_formfactor.npz"))
    return np.concatenate([g["cd_params"], g["se_params"]])


def system(window):
    return systems.make_system("adjoint_0.6nm", RADIUS_NM, N, ms=2, ns=NS, nc=NC, seed=0,
                               elmin=window[0], elmax=window[1])


def run_reference(refbin, S, theta, nthreads):
    tables = {t: O.form_factor_table(theta[4 * t:4 * t + 4], S.vol_per_atom) for t in (0, 1)}
    with tempfile.TemporaryDirectory() as tmp:
        systems.write_reference_inputs(S, tmp, nthreads=nthreads, tables=tables)
        subprocess.run([refbin, str(SEED), str(nthreads)], cwd=tmp, capture_output=True,
                       text=True, check=True)
        ev = np.loadtxt(os.path.join(tmp, "eval.dat"))
    return ev[:, 1], ev[:, 2]


def band_edges(ev_vb, sg_vb, ev_cb, sg_cb):
    v = np.sort(ev_vb[sg_vb < SIGMA_MAX])[-N_VB:]
    c = np.sort(ev_cb[sg_cb < SIGMA_MAX])[:N_CB]
    if len(v) < N_VB or len(c) < N_CB:
        raise RuntimeError("band edges did not converge")
    return np.concatenate([v, c])


def main():
    refdir = build_oracle.build_ref(REF)
    if refdir is None:
        raise SystemExit("the reference checkout (or OpenBLAS) is missing")
    refbin = os.path.join(refdir, "filter_ref")
    nthreads = min(16, os.cpu_count() or 1)
    th0 = theta0()
    S = {k: system(w) for k, w in WINDOWS.items()}

    def edges(theta):
        ev_vb, sg_vb = run_reference(refbin, S["vb"], theta, nthreads)
        ev_cb, sg_cb = run_reference(refbin, S["cb"], theta, nthreads)
        return band_edges(ev_vb, sg_vb, ev_cb, sg_cb), (ev_vb, sg_vb, ev_cb, sg_cb)

    e0, raw = edges(th0)
    print("band edges", e0, flush=True)
    jac = np.zeros((len(e0), len(th0)))
    for j in range(len(th0)):
        tp, tm = th0.copy(), th0.copy()
        tp[j] += H
        tm[j] -= H
        jac[:, j] = (edges(tp)[0] - edges(tm)[0]) / (2 * H)
        print("column", j, jac[:, j], flush=True)
    np.savez_compressed(os.path.join(HERE, "adjoint_ref_fd.npz"), theta=th0, h=H,
                        radius_nm=RADIUS_NM, n=N, ns=NS, nc=NC, seed=SEED,
                        window_vb=np.array(WINDOWS["vb"]), window_cb=np.array(WINDOWS["cb"]),
                        n_vb=N_VB, n_cb=N_CB, sigma_max=SIGMA_MAX, edges=e0, jac_fd=jac,
                        eval_vb=raw[0], sigma_vb=raw[1], eval_cb=raw[2], sigma_cb=raw[3])


if __name__ == "__main__":
    main()
