"""The fused complex64 Newton step in its sub-plane form (cubic grids with
L in {96, 112, 128, 160, 192, 256}): the zy pass (the y transform's R-point stage, z
forward, k^2, z inverse) and the sub-plane pass (the rest of the y transform,
x inverse, epilogue, x forward) against the four line passes that apply the
same operator (filter/hamiltonian.c:27-44, filter/hnorm.c:11-39 inside
filter/filter.c:59-83).

Both paths compute in complex64 with the same DFTs; y and z are split
differently (R x L/R and L/8 x 8 instead of the line passes' N1 x 16), so the
roundings differ.  Tolerance: 2e-5 relative (max over the output) after 40
Newton steps; the FP32 Newton recursion amplifies a rounding difference of one
step by at most the filter's gain, and the 36^3 mixed-precision test bounds
complex64 against FP64 at 1e-4 over 96 steps.
"""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep

pytestmark = pytest.mark.gpu


def _job(L, seed):
    rng = np.random.default_rng(seed)
    dims = (L, L, L)
    n = L ** 3
    steps = (0.7, 0.7, 0.7)
    x = (np.arange(L) - L / 2) * steps[0]
    r2 = x[None, None, :] ** 2 + x[None, :, None] ** 2 + x[:, None, None] ** 2
    pot = (-1.5 * np.exp(-r2 / rng.uniform(20.0, 60.0))).reshape(-1)
    ctx = sep.Context(dims, steps, potl=pot, precision="mixed")
    return ctx, pot, steps[0] ** 3, n


@pytest.mark.parametrize("L", [160, 192, 256])
def test_subplane_step_matches_the_line_passes(L):
    ctx, pot, dv, n = _job(L, L)
    vmin = float(pot.min())
    emax, dE, _ = ctx.energy_range(vmin)
    nc = 40
    ar, ai, zn = sep.coefficients([-1.0, -0.5], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-17, 3, n, dv)
    fused = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_fusion(False)
    lines = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_fusion(True)
    ctx.close()
    rel = np.abs(fused - lines).max() / np.abs(lines).max()
    assert rel < 2e-5, rel
    assert not np.array_equal(fused, np.zeros_like(fused))


def test_subplane_pass_timing_slots():
    """sep_time_passes' last slot times the fused xy pass (the sub-plane pass
    for these grids), and sep_time_fused_step times both passes of the fused
    step; a grid without a fused step reports zeros."""
    ctx, pot, dv, n = _job(160, 3)
    per = ctx.time_passes(2, reps=2)
    fused = ctx.time_fused_step(2, reps=2)
    ctx.close()
    assert len(per) == 7 and per[6] > 0.0
    assert fused[0] > 0.0 and fused[1] > 0.0
    ctx = sep.Context((36, 40, 48), (0.7, 0.7, 0.7), potl=np.zeros(36 * 40 * 48),
                      precision="mixed")
    assert np.array_equal(ctx.time_fused_step(1, reps=1), np.zeros(2))
    ctx.close()


@pytest.mark.parametrize("dims", [(96, 96, 96), (112, 112, 112), (128, 128, 128)])
def test_subplane_form_at_96_to_128_matches_the_line_passes(dims):
    """Cubic 96^3, 112^3 and 128^3 grids take the sub-plane form (y split 4 x 24,
    8 x 14, 4 x 32); grids with nz != nx keep the plane form, which equals the
    line passes bit for bit (tests/test_gpu_batch.py)."""
    ctx, pot, dv, n = _job(dims[0], 5)
    vmin = float(pot.min())
    emax, dE, _ = ctx.energy_range(vmin)
    nc = 40
    ar, ai, zn = sep.coefficients([-1.0, -0.5], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-19, 5, n, dv)
    fused = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_fusion(False)
    lines = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.close()
    rel = np.abs(fused - lines).max() / np.abs(lines).max()
    assert 0.0 < rel < 2e-5, rel
