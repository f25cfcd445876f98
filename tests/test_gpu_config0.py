"""The benchmark's smallest configuration end to end: the 1.2 nm sphere (275
atoms, seeded a0 = +-10 form factors) on its 64^3 grid, 8 start states x 4
targets over [-3.25, -2.95] Ha, nc = 1024 (filter/main.c:64-142).

Against the reference's own program (tests/golden/config0_ref.npz, made by
tests/golden/make_golden.py --config0 from filter/*.c): dE, Vmin, the kept
count, the Ritz values (1e-6 Ha) and sigma.  Against the oracle's FP64 path on
the same inputs: the subspace of the Ritz vectors whose values lie in the
target window (the band-edge subspace of this run) has every principal cosine
>= 0.9999.  The complex64 filter over the full 1023 Newton steps against the
oracle's FP64 filter: the relative error of each filtered state is stated and
bounded (single-precision recursion and accumulation; measured 1e-5..3.5e-5
over the 32 filtered states)."""
import os

import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from oracle import oracle as O
from semi_empirical_pseudopotentials_gb300 import adjoint, systems

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "config0_ref.npz")
E_TOL = 1e-6          # hartree, Ritz values against the reference run
OVERLAP_MIN = 0.9999  # smallest principal cosine of the window subspaces
MIXED_REL = 1e-4      # per filtered state, complex64 vs FP64, 1023 Newton steps


@pytest.fixture(scope="module")
def case():
    g = np.load(GOLD)
    S = systems.make_system("config0", float(g["radius_nm"]), int(g["n"]), int(g["ms"]),
                            int(g["ns"]), int(g["nc"]), seed=int(g["seed"]))
    el = adjoint.window_targets(float(g["elmin"]), float(g["elmax"]), int(g["ms"]))
    nc = int(g["nc"])
    tr = np.zeros((2, 1024))
    tv = np.zeros((2, 1024))
    for t in (0, 1):
        r, v = O.form_factor_table(S.params[t], S.vol_per_atom)
        tr[t], tv[t] = r, O.shift_table(v)
    start = sep.start_states(int(g["start_seed"]), S.ns, S.ngrid, S.dv)
    # GPU, FP64, the whole path with its own energy range
    ctx = sep.Context(S.dims, S.steps, precision="f64")
    pot = ctx.vbuild(S.xyz, S.types.astype(np.int32), tr, tv, [1024, 1024], S.mins)
    vmin = ctx.info()["vmin"]
    res = ctx.pipeline(start, el, nc, vmin, want_psi=True)
    ctx.close()
    # oracle, FP64, the same stages at the reference run's dE
    dE = float(g["dE"])
    dt = (nc / (2.5 * dE)) ** 2
    an_re, _, zn = O.coefficients(el, nc, dE, vmin, dt)
    octx = O.Context(S.dims, pot, O.ksqr(*S.dims, *S.steps), S.dv)
    filt, _ = octx.filter_batch(start, an_re, zn, 4.0 / dE, vmin)
    filt = np.asarray(filt).reshape(S.ns * S.ms, S.ngrid)
    psi = O.normalize_all(filt, S.dv)
    psi, k, _ = octx.portho(psi)
    psi = O.normalize_all(psi[:k], S.dv)
    psi, ev = octx.hmat(psi)
    psi = O.normalize_all(psi, S.dv)
    sg = octx.sigma(psi)
    # GPU complex64 filter on the same start states and coefficients
    cm = sep.Context(S.dims, S.steps, potl=pot, precision="mixed")
    mixed = cm.filter(start, an_re, zn, 4.0 / dE, vmin).reshape(S.ns * S.ms, S.ngrid)
    cm.close()
    return dict(g=g, S=S, el=el, res=res, vmin=vmin, oracle=(ev, sg, psi), filt=filt,
                mixed=mixed)


def test_energy_range_and_vmin_match_reference_run(case):
    g, res = case["g"], case["res"]
    assert abs(res["timing"]["dE"] - float(g["dE"])) <= 1e-9 * float(g["dE"])
    assert case["vmin"] == float(g["vmin"])


def test_ritz_values_and_sigma_match_reference_run(case):
    g, res = case["g"], case["res"]
    assert res["mkept"] == int(g["mkept"])
    assert np.abs(res["eval"] - g["eval"]).max() <= E_TOL
    # eval.dat prints sigma with %g (6 digits)
    assert np.allclose(res["sigma"], g["sigma"], rtol=2e-5, atol=1e-6)


def test_oracle_ritz_values_match_reference_run(case):
    ev, sg, _ = case["oracle"]
    assert len(ev) == int(case["g"]["mkept"])
    assert np.abs(ev - case["g"]["eval"]).max() <= E_TOL


def test_band_edge_subspace_overlap(case):
    S, el, res = case["S"], case["el"], case["res"]
    ev_o, _, psi_o = case["oracle"]
    win_g = (res["eval"] >= el[0]) & (res["eval"] <= el[-1])
    win_o = (ev_o >= el[0]) & (ev_o <= el[-1])
    assert win_g.sum() == win_o.sum() >= 4
    ov = res["psi"][win_g] @ psi_o[win_o].T * S.dv
    cos = np.linalg.svd(ov, compute_uv=False)
    assert cos.min() >= OVERLAP_MIN, cos


def test_mixed_filter_full_length_against_oracle(case):
    f64, f32 = case["filt"], case["mixed"]
    rel = np.linalg.norm(f32 - f64, axis=1) / np.linalg.norm(f64, axis=1)
    print("complex64 vs FP64 filter, relative error per state:", np.array2string(rel, precision=2))
    assert rel.max() <= MIXED_REL, rel
