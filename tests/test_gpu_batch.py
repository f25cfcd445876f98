"""Many nanocrystals in one graph launch, and the tile-shape autotuner.

A batch runs each job's Newton loop as a branch of one CUDA graph: every job's
output must equal that job run alone through sep_filter, bit for bit.  The two
compiled tile shapes split the lines over blocks differently but do the same
arithmetic per line, so the autotuner's choice must not change any result."""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep

pytestmark = pytest.mark.gpu


def _job(dims, seed, precision):
    rng = np.random.default_rng(seed)
    n = int(np.prod(dims))
    steps = (0.9, 0.85, 0.8)
    pot = -1.5 * np.exp(-rng.uniform(0.5, 1.5) * np.linspace(-2, 2, n) ** 2)
    ctx = sep.Context(dims, steps, potl=pot, precision=precision)
    dv = steps[0] * steps[1] * steps[2]
    return ctx, pot, dv, n


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_batch_equals_single_runs(precision):
    # complex64 jobs of (64, 64, 32) run the plane form of the fused step, of
    # (96, 96, 96) the sub-plane form
    shapes = [(32, 32, 32), (36, 40, 48), (48, 48, 48), (64, 64, 32), (96, 96, 96)]
    ns, ms, nc = [3, 4, 2, 3, 2], 3, 40
    jobs = [_job(d, i, precision) for i, d in enumerate(shapes)]
    dE = 40.0
    singles, coefs = [], []
    for (ctx, pot, dv, n), s in zip(jobs, ns):
        vmin = float(pot.min())
        ar, ai, zn = sep.coefficients([-1.2, -0.8, -0.4], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
        start = sep.start_states(-17 - s, s, n, dv)
        singles.append((start, ctx.filter(start, ar, zn, 4.0 / dE, vmin)))
        coefs.append((ar, zn, vmin))
    b = sep.Batch([j[0] for j in jobs], ns, ms, nc)
    for k, (ar, zn, vmin) in enumerate(coefs):
        b.set_coefficients(k, ar, zn, 4.0 / dE, vmin)
        b.load_start(k, singles[k][0])
    b.run()
    for k in range(len(jobs)):
        assert np.array_equal(b.read_out(k), singles[k][1]), k
    b.run()  # the same graph again
    assert np.array_equal(b.read_out(2), singles[2][1])
    b.close()


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_autotuned_tile_shapes_give_identical_results(precision):
    dims = (64, 64, 64)
    ctx, pot, dv, n = _job(dims, 7, precision)
    vmin = float(pot.min())
    nc, dE = 33, 40.0
    ar, ai, zn = sep.coefficients([-1.0, -0.5], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-5, 6, n, dv)
    a = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_tiles([1, 1, 1, 1, 1])
    b = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    assert np.array_equal(a, b)
    choice = ctx.autotune(3, reps=3)
    assert len(choice) == 5 and set(choice) <= {0, 1}
    c = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    assert np.array_equal(a, c)


@pytest.mark.parametrize("dims", [(40, 40, 24), (48, 48, 40), (56, 56, 32), (64, 64, 24),
                                  (96, 96, 24), (128, 128, 16), (72, 72, 128), (80, 80, 128),
                                  (96, 96, 64), (112, 112, 128), (128, 128, 64)])
def test_fused_xy_plane_pass_equals_the_line_passes(dims):
    """The complex64 Newton step with the fused xy plane pass does the same
    arithmetic per line as the four line passes: the filters are equal.  With
    nz = 64 or 128 the 3 pairs have 192 or 384 planes, more than the blocks
    that walk them, so the last y stage of a plane runs fused with the first y
    stage of the next."""
    ctx, pot, dv, npts = _job(dims, 3, "mixed")
    vmin = float(pot.min())
    nc, dE = 70, 40.0
    ar, ai, zn = sep.coefficients([-1.0, -0.6, -0.2], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-11, 5, npts, dv)
    fused = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_fusion(False)
    lines = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_fusion(True)
    d = np.abs(fused - lines).max()
    assert np.array_equal(fused, lines), (d, d / np.abs(lines).max())


@pytest.mark.parametrize("precision,ns", [("mixed", 21), ("f64", 20), ("mixed", 2)])
def test_host_filter_in_chunks_equals_device_filter(precision, ns):
    """sep_filter (host buffers) filters the pairs in a large chunk and a small
    last one, with the copies on their own streams; sep_filter_dev filters all
    pairs at once.  Same arithmetic per pair: the outputs are equal."""
    torch = pytest.importorskip("torch")
    ctx, pot, dv, n = _job((64, 64, 32), 7, precision)
    vmin = float(pot.min())
    nc, dE = 50, 40.0
    ar, ai, zn = sep.coefficients([-1.0, -0.5], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-23, ns, n, dv)
    host = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    sd = torch.from_numpy(start).cuda()
    od = torch.empty((ns, 2, n), dtype=torch.float64, device="cuda")
    ctx.filter_dev(sd.data_ptr(), ns, ar, zn, 4.0 / dE, vmin, od.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(host, od.cpu().numpy())


@pytest.mark.parametrize("dims,K", [((40, 40, 40), 32), ((36, 40, 48), 64)])
def test_two_point_accumulation_equals_the_generic_kernel(dims, K):
    """The complex64 accumulation with 8 targets (k_accumulate_x2: two grid
    points per thread, coefficients read four steps at a time) takes the same
    products in the same order as the generic kernel, which a 9-target filter
    uses: the 8-target filter equals the first 8 targets of the 9-target one
    bit for bit.  nc = 70 leaves a last block of 6 steps (K = 32) or 5 (K =
    64), so the kernels' tails run too."""
    ctx, pot, dv, npts = _job(dims, 4, "mixed")
    ctx.set_block_steps(K)
    vmin = float(pot.min())
    nc, dE = 70, 40.0
    ar, ai, zn = sep.coefficients(np.linspace(-1.2, -0.2, 9), nc, dE, vmin,
                                  (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-13, 5, npts, dv)
    out9 = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    out8 = ctx.filter(start, np.ascontiguousarray(ar[:8]), zn, 4.0 / dE, vmin)
    ctx.close()
    assert np.array_equal(out8, out9[:, :8])
