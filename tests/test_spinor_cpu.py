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
    ref = g["vso_" + form]
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def test_library_rejects_entries_off_the_grid(golden):
    g, nlc = load(golden)
    bad = nlc.copy()
    bad["jxyz"][0, 0] = int(np.prod(g["dims"]))
    with pytest.raises(SepError, match="outside the grid"):
        spinor.nonlocal_potential(g["psi"], bad, g["nl"], float(g["h"]), float(g["h"]) ** 3)
    with pytest.raises(ValueError):
        spinor.nonlocal_potential_kb(g["psi"], nlc, g["nl"], g["elkb"][:1], 1.0)
