"""Spin-orbit operator of the spinor filter (spinors/filterSpinors/): the
oracle against the reference's own init_list, nonlocal_potential and
nonlocal_potential_kb (tests/golden/spinor_vso.npz), and the library's
argument checks.  No GPU needed."""
import numpy as np
import pytest

from oracle import spinor_oracle as so
from semi_empirical_pseudopotentials_gb300 import SepError, spinor


def load(golden):
    g = golden("spinor_vso.npz")
    raw = g["nlc"]
    nlc = raw.reshape(-1).view(so.NLC_DTYPE).reshape(raw.shape[:2])
    return g, nlc


def dense(g, name):
    """The reference's Vso psi: zero away from its stored entries."""
    out = np.zeros(2 * int(np.prod(g["dims"])), dtype=np.complex128)
    out[g[name + "_idx"]] = g[name + "_val"]
    return out


def check_sampled(g, name, got):
    """got (rows x 2N) against the stored samples, sums and sums of squares."""
    got = np.asarray(got).reshape(-1, 2 * int(np.prod(g["dims"])))
    ref = g[name + "_sample"].reshape(got.shape[0], -1)
    scale = np.abs(ref).max()
    assert np.abs(got[:, g["sample_idx"]] - ref).max() <= 1e-12 * scale
    assert np.allclose(got.sum(axis=1), g[name + "_sum"], rtol=1e-11, atol=1e-12 * scale)
    assert np.allclose((np.abs(got) ** 2).sum(axis=1), g[name + "_sumsq"], rtol=1e-11, atol=0)


def test_layouts_match():
    assert so.NLC_DTYPE == spinor.NLC_DTYPE and so.NLC_DTYPE.itemsize == 104


def test_neighbour_lists_match_reference(golden):
    g, ref = load(golden)
    nlc, nl = so.neighbour_lists(g["vx"], g["vy"], g["vz"], g["rxyz"], g["vso"],
                                 float(g["rnlcut2"]), int(g["nnlc"]))
    assert np.array_equal(nl, g["nl"])
    for f in ("jxyz", "y10", "y11", "y1_1", "r", "r2_1", "r2"):
        assert np.array_equal(nlc[f], ref[f]), f
    # exp() of numpy and of the C library may differ in the last bit
    assert np.allclose(nlc["Vr"], ref["Vr"], rtol=4e-16, atol=0)


def test_library_neighbour_lists_match_reference(golden):
    g, ref = load(golden)
    nlc, nl = spinor.neighbour_lists(g["vx"], g["vy"], g["vz"], g["rxyz"], g["vso"],
                                     float(g["rnlcut2"]))
    assert np.array_equal(nl, g["nl"]) and nlc.shape == ref.shape
    for f in ("jxyz", "y10", "y11", "y1_1", "r", "r2_1", "r2", "Vr"):
        assert np.array_equal(nlc[f], ref[f]), f
    with pytest.raises(SepError, match="nnlc is too small"):
        spinor.neighbour_lists(g["vx"], g["vy"], g["vz"], g["rxyz"], g["vso"],
                               float(g["rnlcut2"]), nnlc=int(g["nl"].max()) - 1)


@pytest.mark.parametrize("form", ["gauss", "kb"])
def test_operator_matches_reference(golden, form):
    g, nlc = load(golden)
    n = int(np.prod(g["dims"]))
    h = float(g["h"])
    if form == "gauss":
        got = so.vso_gauss(g["psi"], nlc, g["nl"], h, h ** 3, n)
    else:
        got = so.vso_kb(g["psi"], nlc, g["nl"], g["elkb"], h ** 3, n)
    ref = dense(g, "vso_" + form)
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("form", ["gauss", "kb"])
def test_hamiltonian_matches_reference(golden, form):
    g, nlc = load(golden)
    dims = tuple(int(v) for v in g["dims"])
    h = float(g["h"])
    got = so.hamiltonian(g["psi"], g["potl"], g["ksqr"], dims, nlc, g["nl"], h, h ** 3,
                         flagkb=int(form == "kb"), elkb=g["elkb"])
    check_sampled(g, "h_" + form, got)


def test_newton_filter_matches_reference(golden):
    g, nlc = load(golden)
    dims = tuple(int(v) for v in g["dims"])
    h = float(g["h"])
    got = so.newton_filter(g["psi"], g["an"], g["zn"], float(g["dE_1"]), float(g["vmin"]),
                           g["potl"], g["ksqr"], dims, nlc, g["nl"], h, h ** 3)
    check_sampled(g, "filter_out", got)


def test_library_rejects_entries_off_the_grid(golden):
    g, nlc = load(golden)
    bad = nlc.copy()
    bad["jxyz"][0, 0] = int(np.prod(g["dims"]))
    with pytest.raises(SepError, match="outside the grid"):
        spinor.nonlocal_potential(g["psi"], bad, g["nl"], float(g["h"]), float(g["h"]) ** 3)
    with pytest.raises(ValueError):
        spinor.nonlocal_potential_kb(g["psi"], nlc, g["nl"], g["elkb"][:1], 1.0)


def test_spinor_pipeline_matches_reference(golden):
    """The reference's whole spinor program on the fixture system (energy
    range, coefficients, start states, filtering, portho, Hmat, sigma) against
    the oracle's restatement."""
    from oracle import oracle as O

    g, nlc = load(golden)
    dims = tuple(int(v) for v in g["dims"])
    n = int(np.prod(dims))
    h = float(g["h"])
    dv = h ** 3
    hargs = (g["potl"], g["ksqr"], dims, nlc, g["nl"], h, dv)
    # energy range: init_psi draws four component grids from its fixed seed
    starts = O.start_states(-874917403, 4, n, dv)
    vmin, dE = so.energy_range(list(starts), dv, *hargs)
    assert abs(vmin - float(g["run_vmin"])) <= 1e-9 * abs(float(g["run_vmin"]))
    assert abs(dE - float(g["run_dE"])) <= 1e-9 * float(g["run_dE"])
    # the Newton coefficients are the filter's (complex, both parts used)
    nc = int(g["run_nc"])
    dE_r, vmin_r = float(g["run_dE"]), float(g["run_vmin"])
    ar, ai, zn = O.coefficients(g["run_el"], nc, dE_r, vmin_r, (nc / (2.5 * dE_r)) ** 2)
    assert np.array_equal(ar + 1j * ai, g["run_an"]) and np.array_equal(zn, g["run_zn"])
    # start spinors: consecutive init_psi draws, spin up then down
    ns, ms = int(g["run_ns"]), int(g["run_ms"])
    st = O.start_states(int(g["run_seed"]), 2 * ns, n, dv)
    spinors = [np.concatenate([st[2 * j], st[2 * j + 1]]) for j in range(ns)]
    ev, sig = so.pipeline(spinors, g["run_an"], g["run_zn"], 4.0 / dE_r, vmin_r, dv, *hargs)
    assert len(ev) == int(g["run_mkept"])
    assert np.allclose(ev, g["run_eval"], rtol=1e-9, atol=1e-12)
    assert np.allclose(sig, g["run_sigma"], rtol=1e-7, atol=1e-10)
