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
