"""Band-edge eigenpairs of the complex64 path against the FP64 path, on a case
where both converge: the 1.2 nm CdSe sphere (275 atoms) on its 64^3 grid with
the fitted zb_cdse form factors, one conduction-edge window of 6 targets, 16
start states, nc = 4096 (the whole path of filter/main.c:64-142).

Criteria (per band-edge pair, the 4 lowest conduction states): the FP64 path
reaches sigma <= 1e-5; the complex64 filter followed by the FP64 polish
(sep_ctx_set_polish) gives Ritz values within 1e-6 Ha of the FP64 path's with
sigma <= 1e-5.  Without the polish the complex64 Ritz values already agree
within 1e-6 Ha, while sigma stays above 1e-5 (single-precision rounding noise
in the Ritz vectors)."""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from semi_empirical_pseudopotentials_gb300 import adjoint, systems

pytestmark = pytest.mark.gpu

E_TOL = 1e-6      # hartree, against the FP64 path
SIGMA_MAX = 1e-5  # hartree
N_EDGE = 4
WINDOW = (-0.17, -0.08)


@pytest.fixture(scope="module")
def runs():
    S = systems.make_system("r1.2nm_64_fitted", 1.2, 64, ms=6, ns=16, nc=4096,
                            params=systems.FITTED_CDSE)
    types = S.types.astype(np.int32)
    theta = np.stack([S.params[0], S.params[1]])
    el = adjoint.window_targets(WINDOW[0], WINDOW[1], 6)
    start = sep.start_states(-271828, 16, S.ngrid, S.dv)
    out = {}
    for tag, prec, pol in (("f64", "f64", 0), ("mixed", "mixed", 256),
                           ("mixed_no_polish", "mixed", 0)):
        ctx = sep.Context(S.dims, S.steps, precision=prec)
        ctx.potential_from_params(S.xyz, types, theta, S.vol_per_atom, S.mins)
        ctx.set_polish(pol, 0.01)
        res = ctx.pipeline(start, el, 4096, ctx.info()["vmin"])
        out[tag] = (res["eval"], res["sigma"], res["timing"])
        ctx.close()
    return out


def _edges(ev):
    """The N_EDGE lowest Ritz values at or above the window's lower end (in
    ascending order, so degenerate partners pair one to one)."""
    o = np.argsort(ev)
    return o[ev[o] >= WINDOW[0]][:N_EDGE]


def test_fp64_band_edge_converges(runs):
    ev, sg, _ = runs["f64"]
    idx = _edges(ev)
    assert len(idx) == N_EDGE and sg[idx].max() <= SIGMA_MAX, (ev[idx], sg[idx])


@pytest.mark.parametrize("tag,check_sigma", [("mixed", True), ("mixed_no_polish", False)])
def test_complex64_band_edge_matches_fp64(runs, tag, check_sigma):
    ev, sg, _ = runs["f64"]
    em, sm, t = runs[tag]
    for i, j in zip(_edges(ev), _edges(em)):
        assert abs(em[j] - ev[i]) <= E_TOL, (tag, ev[i], em[j])
        if check_sigma:
            assert sm[j] <= SIGMA_MAX, (tag, ev[i], sm[j])
    if tag == "mixed":
        assert t["polish_s"] > 0.0
