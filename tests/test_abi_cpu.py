"""C ABI checks that need no GPU: the library loads, exports every function
that include/*.h declares, and its host numerics match the reference's own
outputs bit for bit (tests/golden, made from the reference's sources)."""
import ctypes
import os
import re

import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from semi_empirical_pseudopotentials_gb300 import binding

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sep_[a-z0-9_]+|[a-zA-Z_]\w*)\s*\(", text)) -
                  {"if", "sizeof", "defined"})


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(binding.LIB_PATH)
    names = [n for n in declared("sep_gb300.h") if n.startswith("sep_")]
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_fd_compat_exports():
    path = os.path.join(os.path.dirname(binding.LIB_PATH), "libsep_fdcompat.so")
    if not os.path.exists(os.path.join(ROOT, "include", "sep_fd_compat.h")):
        pytest.skip("no fd compat header")
    lib = ctypes.CDLL(path)
    for n in declared("sep_fd_compat.h"):
        if n in ("zomplex",):
            continue
        assert hasattr(lib, n), n


def test_no_device_is_reported_cleanly():
    n = sep.device_count()
    assert n >= 0
    if n == 0:
        with pytest.raises(sep.SepError):
            sep.Context((16, 16, 16), (0.5, 0.5, 0.5))


@pytest.mark.parametrize("nc", [128, 1024])
def test_coefficients_bit_exact(golden, nc):
    g = golden("ref_small.npz")
    ar, ai, zn = sep.coefficients(g["el"], nc, float(g["dE"]), float(g["vmin"]),
                                  float(g[f"dt_{nc}"]))
    assert np.array_equal(zn, g[f"zn_{nc}"])
    assert np.array_equal(ar, g[f"an_{nc}"].real)
    assert np.array_equal(ai, g[f"an_{nc}"].imag)


def test_start_states_bit_exact(golden):
    g = golden("ref_small.npz")
    n = int(np.prod(g["dims"]))
    got = sep.start_states(-777, 2, n, float(g["dv"]))
    assert np.array_equal(got, g["init_psi_seed777"])


def test_ksqr_bit_exact(golden):
    g = golden("ref_small.npz")
    got = sep.ksqr(tuple(int(v) for v in g["dims"]), (g["dx"], g["dy"], g["dz"]))
    assert np.array_equal(got, g["ksqr"])


def test_form_factor_table(golden):
    g = golden("zb_cdse_formfactor.npz")
    for key, pot in (("cd_params", g["pot_cd"]), ("se_params", g["pot_se"])):
        r, v = sep.form_factor_table(g[key], float(g["vol_per_atom"]))
        assert np.allclose(r, pot[:, 0], rtol=6e-6, atol=1e-12)
        assert np.allclose(v, pot[:, 1], rtol=6e-6, atol=6e-6 * np.abs(pot[:, 1]).max())
    # and bit-identical to the tables the reference read in ref_small
    s = golden("ref_small.npz")
    for t in range(2):
        r, v = sep.form_factor_table(s["params"][t], float(s["vol_per_atom"]))
        assert np.array_equal(r, s["tab_r"][t]) and np.array_equal(v, s["tab_v"][t])


def test_bad_arguments_raise():
    with pytest.raises(sep.SepError):
        sep.coefficients([0.1], 0, 1.0, 0.0, 1.0)
    with pytest.raises(sep.SepError):
        sep.start_states(-1, 0, 10, 1.0)


def test_form_factor_backward_matches_central_differences():
    """sep_form_factor_backward (shift adjoint + sine-transform Jacobian) against
    central differences of w . shifted_table(a), all on the host."""
    a = np.array([10.2, 1.45, 29.0, 0.31])
    vol = 189.6
    w = np.random.default_rng(0).standard_normal(1024)

    def L(p):
        v = sep.form_factor_table(p, vol)[1]
        return float(w @ (v - v[-1]))

    g = sep.form_factor_backward(a, vol, w)
    for j in range(4):
        h = 1e-6 * max(1.0, abs(a[j]))
        ap, am = a.copy(), a.copy()
        ap[j] += h
        am[j] -= h
        fd = (L(ap) - L(am)) / (2 * h)
        assert abs(fd - g[j]) <= 1e-6 * np.abs(g).max(), (j, fd, g[j])


def test_band_edge_selection():
    from semi_empirical_pseudopotentials_gb300 import adjoint

    ev = np.array([-0.5, -0.45, -0.44, -0.43, -0.42, -0.2, -0.19, -0.18, -0.17, -0.1, 0.3])
    sg = np.full_like(ev, 1e-8)
    sg[-1] = 1.0
    idx = adjoint.select_band_edges(ev, sg, 4)
    assert list(ev[idx]) == [-0.45, -0.44, -0.43, -0.42, -0.2, -0.19, -0.18, -0.17]
