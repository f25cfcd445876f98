"""The large-grid workload's path (the 4 nm sphere on a 192^3 grid) on a small
case: the Newton filter at length 192 in both precisions (FP64 line passes;
complex64 in the sub-plane form of the fused step) against the oracle
(filter/filter.c:59-83), and the pipeline (filter/main.c:64-142) when the
device is short of memory, which releases the filter's workspaces before
ortho.

Tolerances: FP64 filter 1e-9 relative; complex64 filter 1e-4 relative over
16 Newton steps (FP32 rounding in the recursion, as the 36^3 mixed test);
the pipeline with and without the release: identical Ritz values (the same
kernels on the same inputs).
"""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DIMS = (192, 192, 192)


def _smooth_system(dims, seed):
    rng = np.random.default_rng(seed)
    steps = (0.7, 0.65, 0.6)
    nx, ny, nz = dims
    x = np.arange(nx) * steps[0]
    y = np.arange(ny) * steps[1]
    z = np.arange(nz) * steps[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    v = np.zeros_like(X)
    for _ in range(6):
        c = rng.uniform(0, 1, 3) * np.array([x[-1], y[-1], z[-1]])
        a = rng.uniform(-2, 2)
        v += a * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / 4.0)
    return steps, v.reshape(-1)


@pytest.fixture(scope="module")
def case():
    steps, pot = _smooth_system(DIMS, seed=7)
    n = int(np.prod(DIMS))
    dv = steps[0] * steps[1] * steps[2]
    vmin = float(pot.min())
    ctx64 = sep.Context(DIMS, steps, potl=pot, precision="f64")
    emax, dE, _ = ctx64.energy_range(vmin)
    nc = 16
    ar, ai, zn = O.coefficients([-1.0, 0.0], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = O.start_states(-77, 2, n, dv)
    octx = O.Context(DIMS, pot, O.ksqr(*DIMS, *steps), dv)
    ref = np.stack([octx.filter_cycle(start[s], ar, zn, 4.0 / dE, vmin) for s in range(2)])
    return dict(steps=steps, pot=pot, dv=dv, vmin=vmin, dE=dE, ar=ar, zn=zn, start=start,
                ref=ref, ctx64=ctx64)


def test_fp64_filter_at_192_matches_oracle(case):
    got = case["ctx64"].filter(case["start"], case["ar"], case["zn"], 4.0 / case["dE"],
                               case["vmin"])
    rel = np.linalg.norm(got - case["ref"]) / np.linalg.norm(case["ref"])
    assert rel < 1e-9, rel


def test_complex64_filter_at_192_matches_oracle(case):
    ctx = sep.Context(DIMS, case["steps"], potl=case["pot"], precision="mixed")
    got = ctx.filter(case["start"], case["ar"], case["zn"], 4.0 / case["dE"], case["vmin"])
    ctx.close()
    rel = np.linalg.norm(got - case["ref"]) / np.linalg.norm(case["ref"])
    assert rel < 1e-4, rel


def test_pipeline_releases_filter_workspace_when_short(case):
    """ortho needs 8 n m bytes for a second block of states plus about 6 GB of
    contraction workspace; with less free memory than that the pipeline drops
    the filter's workspaces first.  The results do not change."""
    torch = pytest.importorskip("torch")
    n = int(np.prod(DIMS))
    ns, el, nc = 4, np.array([-1.0, -0.5]), 32
    start = O.start_states(-91, ns, n, case["dv"])
    ctx = sep.Context(DIMS, case["steps"], potl=case["pot"], precision="mixed")
    a = ctx.pipeline(start, el, nc, case["vmin"], dE=case["dE"])
    need = 8 * n * ns * len(el) + (6 << 30)
    free, _ = torch.cuda.mem_get_info()
    # hold all but about 2 GB less than ortho asks for
    hog = torch.empty(max(0, free - need + (2 << 30)), dtype=torch.uint8, device="cuda")
    assert torch.cuda.mem_get_info()[0] < need
    b = ctx.pipeline(start, el, nc, case["vmin"], dE=case["dE"])
    del hog
    torch.cuda.empty_cache()
    ctx.close()
    assert a["mkept"] == b["mkept"] > 0
    assert np.array_equal(a["eval"], b["eval"])
    assert np.array_equal(a["sigma"], b["sigma"])
