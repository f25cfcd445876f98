"""Spin-orbit operator of the spinor filter on the GPU (sep_spinor_vso,
through the C ABI) against the reference's own outputs
(tests/golden/spinor_vso.npz) and the oracle (oracle/spinor_oracle.py)."""
import ctypes as C

import numpy as np
import pytest

from oracle import spinor_oracle as so
from semi_empirical_pseudopotentials_gb300 import binding, spinor

pytestmark = pytest.mark.gpu


def load(golden):
    g = golden("spinor_vso.npz")
    raw = g["nlc"]
    return g, raw.reshape(-1).view(so.NLC_DTYPE).reshape(raw.shape[:2])


@pytest.mark.parametrize("form", ["gauss", "kb"])
def test_matches_reference_outputs(golden, form):
    g, nlc = load(golden)
    h = float(g["h"])
    if form == "gauss":
        got = spinor.nonlocal_potential(g["psi"], nlc, g["nl"], h, h ** 3)
    else:
        got = spinor.nonlocal_potential_kb(g["psi"], nlc, g["nl"], g["elkb"], h ** 3)
    ref = np.zeros_like(got)
    ref[g["vso_" + form + "_idx"]] = g["vso_" + form + "_val"]
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def overlapping_case(seed=3, n=40, h=0.5, natom=24):
    """40^3 grid, 24 atoms whose neighbourhoods overlap (the contributions of
    several atoms add on shared points)."""
    rng = np.random.default_rng(seed)
    v = -0.5 * n * h + h * np.arange(n)
    rxyz = rng.uniform(-6.0, 6.0, size=(natom, 3))
    nlc, nl = so.neighbour_lists(v, v, v, rxyz, rng.uniform(-0.1, 0.1, natom),
                                 0.49 * 6.0 * np.log(10.0), 700)
    nlc["Vs0G1"] = rng.normal(size=nlc.shape)
    nlc["Vs0G_2"] = rng.normal(size=nlc.shape)
    psi = rng.normal(size=2 * n ** 3) + 1j * rng.normal(size=2 * n ** 3)
    return nlc, nl, psi, rng.uniform(0.5, 2.0, 2 * natom), h, n ** 3


def test_overlapping_atoms_match_oracle():
    nlc, nl, psi, elkb, h, ng = overlapping_case()
    ref = so.vso_gauss(psi, nlc, nl, h, h ** 3, ng)
    got = spinor.nonlocal_potential(psi, nlc, nl, h, h ** 3)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    ref = so.vso_kb(psi, nlc, nl, elkb, h ** 3, ng)
    got = spinor.nonlocal_potential_kb(psi, nlc, nl, elkb, h ** 3)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_device_entry_point_on_a_stream():
    torch = pytest.importorskip("torch")
    nlc, nl, psi, elkb, h, ng = overlapping_case(seed=5)
    dev = torch.device("cuda:0")
    d_psi = torch.from_numpy(psi.view(np.float64).copy()).to(dev)
    d_nlc = torch.from_numpy(np.ascontiguousarray(nlc).view(np.uint8).reshape(-1).copy()).to(dev)
    d_nl = torch.from_numpy(nl.astype(np.int64)).to(dev)
    d_out = torch.empty_like(d_psi)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        st = binding.lib().sep_spinor_vso_dev(
            C.c_void_p(d_psi.data_ptr()), ng, nlc.shape[0], nlc.shape[1],
            C.c_void_p(d_nlc.data_ptr()), C.c_void_p(d_nl.data_ptr()), h, h ** 3, 0, None,
            C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == 0
    stream.synchronize()
    got = d_out.cpu().numpy().view(np.complex128)
    ref = spinor.nonlocal_potential(psi, nlc, nl, h, h ** 3)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
