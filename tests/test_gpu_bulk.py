"""Bulk band structures and their gradient on the GPU (sep_bulk_*, through
the C ABI) against the oracle (oracle/bulk_oracle.py) and the reference's
published runs (tests/golden/bulk_fit.json)."""
import numpy as np
import pytest

from oracle import bulk_oracle as bo
from semi_empirical_pseudopotentials_gb300 import bulk
from tests import fixture_bulk as fb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fits(tmp_path_factory):
    return {run: bulk.read_fit_inputs(fb.materialise(run, str(tmp_path_factory.mktemp(run))))
            for run in ("zb_cdse", "w_cdse", "cdse")}


@pytest.mark.parametrize("run,i", [("zb_cdse", 0), ("w_cdse", 0), ("cdse", 1)])
def test_bands_match_oracle_and_published(fits, golden, run, i):
    c = fits[run].crystals[i]
    bc = bulk.BulkCrystal(c, fits[run].ke_scale)
    p = bc.type_params(fb.best_atom_params(run)[i])
    got = bc.bands(p)
    ref = bo.bands(c.cell, c.tau, fb.best_atom_params(run)[i], c.kpts, c.max_ke, c.ne,
                   fits[run].ke_scale)
    assert np.abs(got - ref).max() < 1e-8                # eV
    assert np.abs(got - fb.published_bands(run, i)[1]).max() < 1.2e-5
    # the reference's own calcBandStructure in full precision
    full = golden("bulk_ref.npz")[f"{run}_bands"]
    off = sum(cc.ne * len(cc.kpts) for cc in fits[run].crystals[:i])
    mine = full[off:off + c.ne * len(c.kpts)].reshape(len(c.kpts), c.ne)
    assert np.abs(got - mine).max() < 1e-8
    bc.close()


def test_solver_paths_agree(fits):
    """The library's batched solver (default), cuSOLVER's batched routine and
    cuSOLVER one matrix per call give the same bands and the same gradient."""
    c = fits["w_cdse"].crystals[0]
    bc = bulk.BulkCrystal(c)
    p = bc.type_params(fb.best_atom_params("w_cdse")[0])
    rng = np.random.default_rng(4)
    dl = rng.uniform(-1.0, 1.0, (bc.nk, bc.nev))
    a, ga = bc.backward(p, dl)
    assert bc.solver_path == 2
    bc.set_eigensolver("cusolver")
    b, gb = bc.backward(p, dl)
    assert bc.solver_path in (0, 1)
    bc.set_solver(False)
    c2 = bc.bands(p)
    assert bc.solver_path == 0
    assert np.abs(a - b).max() < 1e-9
    assert np.abs(a - c2).max() < 1e-9
    # the gradient (eigenvectors, degenerate clusters by perturbation theory)
    assert np.abs(ga - gb).max() <= 1e-8 * max(1.0, np.abs(gb).max())
    bc.close()


def cluster_weights(e_full, nev, rng):
    """Per k-point weights that are equal inside each cluster of degenerate
    bands (so that the weighted sum of bands is differentiable); a cluster
    that reaches past band nev gets weight 0."""
    w = np.zeros((e_full.shape[0], nev))
    for k in range(e_full.shape[0]):
        n = 0
        while n < nev:
            m = n + 1
            while m < e_full.shape[1] and e_full[k, m] - e_full[k, m - 1] < 1e-3:
                m += 1
            if m <= nev:
                w[k, n:m] = rng.uniform(0.5, 1.5)
            n = m
    return w


# the oracle's differences for every parameter of zb_cdse, for a0 of each
# element of w_cdse (one oracle evaluation there takes about a second)
@pytest.mark.parametrize("run,oracle_params", [("zb_cdse", (0, 1, 2, 3)), ("w_cdse", (0,))])
def test_gradient_matches_reference_derived_differences(fits, run, oracle_params):
    c = fits[run].crystals[0]
    bc = bulk.BulkCrystal(c)
    atom_p = fb.best_atom_params(run)[0]
    p = bc.type_params(atom_p)
    full = bo.bands(c.cell, c.tau, atom_p, c.kpts, c.max_ke, c.ne + 2)
    w = cluster_weights(full, c.ne, np.random.default_rng(7))
    _, grad = bc.backward(p, w)
    types = [bc.types_of.index(s) for s in c.symbols]

    def loss_oracle(pp):
        return float(np.sum(w * bo.bands(c.cell, c.tau, pp[types], c.kpts, c.max_ke, c.ne)))

    def loss_gpu(pp):
        return float(np.sum(w * bc.bands(pp)))

    # with h = 1e-6 the bands move by about 1e-4 eV, far less than the 1 meV
    # that separates the weight clusters
    h = 1e-6
    fd_ref, fd_gpu = np.full_like(p, np.nan), np.zeros_like(p)
    for t in range(p.shape[0]):
        for m in range(4):
            e = np.zeros_like(p)
            e[t, m] = h
            fd_gpu[t, m] = (loss_gpu(p + e) - loss_gpu(p - e)) / (2 * h)
            if m in oracle_params:
                fd_ref[t, m] = (loss_oracle(p + e) - loss_oracle(p - e)) / (2 * h)
    scale = np.abs(fd_gpu).max()
    sel = ~np.isnan(fd_ref)
    assert np.abs(grad - fd_ref)[sel].max() < 1e-6 * scale, (grad, fd_ref)
    assert np.abs(grad - fd_gpu).max() < 1e-6 * scale, (grad, fd_gpu)
    bc.close()


def test_fit_objective_and_gradient(fits):
    fit = fits["cdse"]
    bf = bulk.BulkFit(fit)
    best = fb.best_atom_params("cdse")
    theta = np.array([best[0][0], best[0][2]])
    val, grad = bf.objective_and_grad(theta)
    # the oracle's objective (fit.c:101-122) on the same crystal parameters
    ref = np.mean([bo.weighted_mse(
        bo.bands(c.cell, c.tau, [bulk.fit_atom_params(fit, theta, ci, s) for s in c.symbols],
                 c.kpts, c.max_ke, c.ne), c.exp_bands) for ci, c in enumerate(fit.crystals)])
    assert abs(val - ref) < 1e-9 * ref
    assert abs(bf.objective(theta) - val) < 1e-12 * val
    # the chain to the shared parameters: sum of each crystal's gradient
    manual = np.zeros_like(theta)
    for ci, (bc, p) in enumerate(zip(bf.crystals, bf.crystal_params(theta))):
        b = bc.bands(p)
        _, d = bf._mse_terms(ci, b)
        _, gp = bc.backward(p, d / len(bf.crystals))
        for t, s in enumerate(bc.types_of):
            f = gp[t].copy()
            if ci == 1:
                f[0] *= fit.norm_vol[1] / fit.norm_vol[0]
            manual[fit.elements.index(s)] += f
    assert np.allclose(grad, manual, rtol=1e-12, atol=0)
    torch = pytest.importorskip("torch")
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    loss = bulk.BandStructureMSE.apply(th, bf)
    loss.backward()
    assert abs(loss.item() - val) < 1e-12 * val
    assert np.allclose(th.grad.numpy(), grad, rtol=1e-12, atol=0)
    bf.close()


def test_bad_arguments_are_reported():
    with pytest.raises(bulk.SepError):
        bulk.basis(np.zeros(9), 5.0)
    c = bulk.Crystal(cell=np.eye(3) * 10.0, symbols=["X"], tau=np.zeros((1, 3)),
                     kpts=np.zeros((1, 3)), max_ke=1.0, ne=10 ** 6, scale=10.0)
    with pytest.raises(bulk.SepError):
        bulk.BulkCrystal(c)


def test_fit_driver_on_the_gpu(tmp_path):
    d = fb.materialise("zb_cdse", str(tmp_path / "run"))
    fit = bulk.read_fit_inputs(d)
    bf = bulk.BulkFit(fit)
    start = bf.objective(fit.params)
    bf.close()
    theta, best = bulk.run_fit(d, steps=3, lr=1e-3)
    assert best <= start * (1 + 1e-9)
    for name in ("iterations.dat", "output.dat", "bandStruct_0.dat", "kpoints_0.dat",
                 "pot_Cd_0.dat", "best_Se_0_Params.dat"):
        assert (tmp_path / "run" / name).exists(), name


@pytest.mark.parametrize("run", ["zb_cdse", "w_cdse"])
def test_fit_objective_gradient_with_real_weights_matches_central_differences(fits, run):
    """The fit objective (fit.c:101-122) with its real band weights
    (fit.c:106-112), whose weights differ inside degenerate clusters (the
    valence-band top at Gamma): the gradient equals central differences of
    the objective on the GPU (every parameter) and of the oracle's objective
    (a0 of each element), h = 1e-6, within 1e-6 of the largest entry."""
    fit = fits[run]
    bf = bulk.BulkFit(fit)
    theta = np.asarray(fit.params, dtype=np.float64)
    _, grad = bf.objective_and_grad(theta)

    def oracle_objective(th):
        return np.mean([bo.weighted_mse(
            bo.bands(c.cell, c.tau, [bulk.fit_atom_params(fit, th, ci, s) for s in c.symbols],
                     c.kpts, c.max_ke, c.ne, fit.ke_scale), c.exp_bands)
            for ci, c in enumerate(fit.crystals)])

    h = 1e-6
    flat = theta.reshape(-1)
    fd, fd_ref = np.zeros(flat.size), np.full(flat.size, np.nan)
    for j in range(flat.size):
        e = np.zeros(flat.size)
        e[j] = h
        tp, tm = (flat + e).reshape(theta.shape), (flat - e).reshape(theta.shape)
        fd[j] = (bf.objective(tp) - bf.objective(tm)) / (2 * h)
        if j % 4 == 0:
            fd_ref[j] = (oracle_objective(tp) - oracle_objective(tm)) / (2 * h)
    g = grad.reshape(-1)
    scale = np.abs(fd).max()
    assert np.abs(g - fd).max() < 1e-6 * scale, (g, fd)
    sel = ~np.isnan(fd_ref)
    assert np.abs(g - fd_ref)[sel].max() < 1e-6 * scale, (g, fd_ref)
    bf.close()
