"""Bulk band-structure path (pseudopotFitting/) on the CPU: the input readers,
the plane-wave basis of the native library, and the oracle against the
reference's published runs (tests/golden/bulk_fit.json)."""
import numpy as np
import pytest

from oracle import bulk_oracle as bo
from semi_empirical_pseudopotentials_gb300 import bulk
from tests import fixture_bulk as fb


@pytest.fixture(scope="module")
def fits(tmp_path_factory):
    out = {}
    for run in ("zb_cdse", "w_cdse", "cdse"):
        d = fb.materialise(run, str(tmp_path_factory.mktemp(run)))
        out[run] = bulk.read_fit_inputs(d)
    return out


def test_reader_follows_the_reference(fits):
    zb = fits["zb_cdse"].crystals[0]
    # TESTS/zb_cdse/run.dat: "Cell 0 volume = 375.13616804"; output.dat: Cd at 1.43107
    assert abs(zb.volume - 375.13616804) < 5e-9
    assert np.allclose(zb.tau, [[1.43107] * 3, [-1.43107] * 3], atol=5e-6)
    assert zb.symbols == ["Cd", "Se"] and zb.ne == 8 and len(zb.kpts) == 20
    w = fits["w_cdse"].crystals[0]
    assert w.symbols == ["Cd", "Cd", "Se", "Se"] and w.ne == 16 and len(w.kpts) == 42
    two = fits["cdse"]
    assert [len(c.kpts) for c in two.crystals] == [42, 20] and two.elements == ["Cd", "Se"]


@pytest.mark.parametrize("run,counts", [("zb_cdse", [199]), ("w_cdse", [377]),
                                        ("cdse", [377, 387])])
def test_basis_size_matches_output_dat(fits, run, counts):
    # output.dat: "The number of basis functions used was: N"
    got = [len(bulk.basis(c.cell, c.max_ke)) for c in fits[run].crystals]
    assert got == counts


def test_basis_matches_oracle(fits):
    c = fits["w_cdse"].crystals[0]
    g = bulk.basis(c.cell, c.max_ke)
    ref = bo.basis(c.cell, c.max_ke)
    mag = np.sqrt((g * g).sum(1))
    assert np.all(np.diff(mag) >= 0)
    key = lambda a: sorted(map(tuple, np.round(a, 9)))
    assert key(g) == key(ref)


def test_a0_volume_scaling_matches_output_dat(fits):
    # cdse: the zincblende crystal's a0 is the wurtzite one's times the ratio
    # of volumes per atom (init.c:72-80); output.dat prints both
    fit = fits["cdse"]
    best = fb.best_atom_params("cdse")
    theta = np.array([best[0][0], best[0][2]])          # Cd, Se of crystal 0
    for a, s in enumerate(fit.crystals[1].symbols):
        got = bulk.fit_atom_params(fit, theta, 1, s)
        assert np.allclose(got, best[1][a], rtol=0, atol=6e-9), s


@pytest.mark.parametrize("run,i", [("zb_cdse", 0), ("w_cdse", 0), ("cdse", 0), ("cdse", 1)])
def test_oracle_matches_published_band_structures(fits, run, i):
    c = fits[run].crystals[i]
    kmag, pub = fb.published_bands(run, i)
    params = fb.best_atom_params(run)[i]
    b = bo.bands(c.cell, c.tau, params, c.kpts, c.max_ke, c.ne, fits[run].ke_scale)
    # 5 printed decimals; the parameters printed with 8
    assert np.abs(b - pub).max() < 1.2e-5
    assert np.abs(np.sqrt((c.kpts ** 2).sum(1)) - kmag).max() < 5.1e-6


def test_unweighted_mse_matches_published(fits):
    # w_cdse/output.dat: "The best mean squared error found was:  0.14712"
    c = fits["w_cdse"].crystals[0]
    _, pub = fb.published_bands("w_cdse", 0)
    use = np.abs(c.exp_bands) > 1e-10
    assert abs(np.mean((pub - c.exp_bands)[use] ** 2) - 0.14712) < 5e-6


def test_band_weights():
    assert list(bulk.band_weights(8)) == [0.06125, 2, 4, 4, 4, 4, 2, 0.06125]
    assert np.array_equal(bulk.band_weights(16), bo.band_weights(16))


def test_band_structure_file_format(fits, tmp_path):
    c = fits["zb_cdse"].crystals[0]
    _, pub = fb.published_bands("zb_cdse", 0)
    bulk.write_band_structure(tmp_path / "bandStruct_0.dat", c.kpts, pub)
    got = (tmp_path / "bandStruct_0.dat").read_text().splitlines()
    want = fb.runs()["zb_cdse"]["bandStucture_0.dat"].splitlines()
    # the band columns are byte-identical; |k| is recomputed
    assert [g.split(" ", 2)[2] for g in got] == [w.split(" ", 2)[2] for w in want]


class StubFit:
    """Stands in for BulkFit in the driver's host logic: a quadratic
    objective, and the oracle's band structures."""

    def __init__(self, fit):
        self.fit = fit
        self.target = np.asarray(fit.params) * 1.01
        self.crystals = [type("C", (), {"nbv": len(bo.basis(c.cell, c.max_ke))})()
                         for c in fit.crystals]

    def objective_and_grad(self, theta):
        d = theta - self.target
        return float(np.sum(d * d)), 2.0 * d

    def band_structures(self, theta):
        f = self.fit
        return [bo.bands(c.cell, c.tau, [bulk.fit_atom_params(f, theta, ci, s) for s in c.symbols],
                         c.kpts, c.max_ke, c.ne, f.ke_scale) for ci, c in enumerate(f.crystals)]


def test_fit_driver_writes_the_reference_files(tmp_path):
    d = fb.materialise("zb_cdse", str(tmp_path / "run"))
    pub = fb.runs()["zb_cdse"]
    theta, best = bulk.run_fit(d, steps=0, fitter=StubFit)   # input.par: nIterations 0
    out = lambda name: open(f"{d}/{name}").read()
    # the inputs' k-points and real-space tables, byte for byte (write.c:155-160, pot.c:73-77)
    assert out("kpoints_0.dat") == pub["kpoints_0.dat"]
    assert out("pot_Cd_0.dat") == pub["pot_Cd_0.dat"]
    assert out("pot_Se_0.dat") == pub["pot_Se_0.dat"]
    # the parameter block of output.dat as the reference printed it
    block = pub["output.dat"].split("The best mean squared error found was:")[1]
    block = block.split("\n", 1)[1].split("*****")[0].rstrip()
    assert block in out("output.dat")
    assert "The number of basis functions used was: 199\n" in out("output.dat")
    assert out("best_Cd_0_Params.dat") == " 0.04248460\n 0.67188400\n 0.13608200\n 0.51454400\n"
    got = np.loadtxt(f"{d}/bandStruct_0.dat")[:, 1:]
    assert np.abs(got - fb.published_bands("zb_cdse", 0)[1]).max() < 2e-5


def test_fit_driver_iterations_log(tmp_path):
    d = fb.materialise("zb_cdse", str(tmp_path / "run"))
    theta, best = bulk.run_fit(d, steps=20, lr=0.002, fitter=StubFit)
    log = open(f"{d}/iterations.dat").read()
    assert [l for l in log.splitlines() if l.startswith("Iteration")] == \
        ["Iteration 0", "Iteration 10", "Iteration 20"]
    mses = [float(l.split()[1]) for l in log.splitlines() if l.startswith("MSE")]
    assert mses[-1] < mses[0]
    fit = bulk.read_fit_inputs(d)
    assert best < float(np.sum((fit.params - fit.params * 1.01) ** 2))


# full-precision pins against the reference's own compiled code
# (tests/golden/bulk_ref.npz, from tests/golden/make_bulk_fixture.py)
@pytest.mark.parametrize("run", ["zb_cdse", "w_cdse", "cdse"])
def test_oracle_bands_and_objectives_match_reference_code(fits, golden, run):
    ref = golden("bulk_ref.npz")
    fit = fits[run]
    best = fb.best_atom_params(run)
    bands = [bo.bands(c.cell, c.tau, best[i], c.kpts, c.max_ke, c.ne, fit.ke_scale)
             for i, c in enumerate(fit.crystals)]
    assert np.abs(np.concatenate([b.ravel() for b in bands]) - ref[f"{run}_bands"]).max() < 1e-10
    # the fit objective of BulkFit (host arithmetic) on the reference's bands
    stub = type("S", (), {"fit": fit})()
    off, terms_w, terms = 0, [], []
    for i, c in enumerate(fit.crystals):
        n = c.ne * len(c.kpts)
        b = ref[f"{run}_bands"][off:off + n].reshape(len(c.kpts), c.ne)
        off += n
        terms_w.append(bulk.BulkFit._mse_terms(stub, i, b, True)[0])
        terms.append(bulk.BulkFit._mse_terms(stub, i, b, False)[0])
    assert abs(np.mean(terms_w) - float(ref[f"{run}_weighted_mse"])) <= 1e-13 * np.mean(terms_w)
    assert abs(np.mean(terms) - float(ref[f"{run}_mse"])) <= 1e-13 * np.mean(terms)


@pytest.mark.parametrize("run", ["zb_cdse", "cdse"])
def test_basis_matches_reference_code(fits, golden, run):
    ref = golden("bulk_ref.npz")
    for i, c in enumerate(fits[run].crystals):
        g = bulk.basis(c.cell, c.max_ke)
        r = ref[f"{run}_basis_{i}"]
        assert len(g) == int(ref[f"{run}_nbv_{i}"]) == len(r)
        key = lambda a: sorted(map(tuple, np.round(a, 10)))
        assert key(g) == key(r)
        # the same shells in the same order of |G|
        assert np.allclose(np.sqrt((g * g).sum(1)), np.sqrt((r * r).sum(1)), rtol=0, atol=1e-12)
