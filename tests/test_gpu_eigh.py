"""The library's FP64 symmetric eigensolver (sep_eigh; Householder
tridiagonalisation, divide and conquer, back-transformation) against
numpy.linalg.eigh, and the whole filter path with it in place of cuSOLVER.

Tolerances, with ||A|| the largest |eigenvalue|: eigenvalues within
1e-13 n ||A|| of LAPACK's; residuals ||A v - w v|| <= 1e-13 n ||A||;
||V^T V - I||_max <= 1e-13 n."""
import ctypes as C

import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from semi_empirical_pseudopotentials_gb300 import binding

pytestmark = pytest.mark.gpu


def eigh(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = a.shape[0]
    w = np.empty(n)
    v = np.empty((n, n))
    L = binding.lib()
    L.sep_eigh.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]
    binding._check(L.sep_eigh(a.ctypes.data, n, w.ctypes.data, v.ctypes.data))
    return w, v.T  # column-major output: columns are the eigenvectors


def check(a, w, v):
    n = a.shape[0]
    ref = np.linalg.eigvalsh(a)
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.all(np.diff(w) >= -1e-13 * scale)
    assert np.abs(w - ref).max() <= 1e-13 * n * scale, np.abs(w - ref).max() / scale
    res = np.abs(a @ v - v * w[None, :]).max()
    assert res <= 1e-13 * n * scale, res / scale
    orth = np.abs(v.T @ v - np.eye(n)).max()
    assert orth <= 1e-13 * n, orth


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 9, 17, 32, 33, 64, 100, 257, 512, 1000])
def test_random_symmetric(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    a = a + a.T
    check(a, *eigh(a))


def spectrum_matrix(lam, seed):
    n = len(lam)
    q, _ = np.linalg.qr(np.random.default_rng(seed).standard_normal((n, n)))
    return (q * lam[None, :]) @ q.T


@pytest.mark.parametrize("case", ["degenerate", "graded", "clustered"])
def test_hard_spectra(case):
    rng = np.random.default_rng(7)
    n = 300
    if case == "degenerate":   # multiplicities 1..6, as symmetric Ritz problems have
        lam = np.repeat(rng.uniform(-2, 2, 70), rng.integers(1, 7, 70))[:n]
        lam = np.concatenate([lam, rng.uniform(-2, 2, n - len(lam))])
    elif case == "graded":     # 1 .. 1e-20, as a Gram matrix of filtered states
        lam = np.logspace(0, -20, n)
    else:                      # dense clusters 1e-9 wide
        lam = np.concatenate([c + 1e-9 * rng.standard_normal(30) for c in rng.uniform(-1, 1, 10)])
    a = spectrum_matrix(np.sort(lam), 11)
    a = 0.5 * (a + a.T)
    check(a, *eigh(a))


def test_gram_matrix_of_dependent_vectors():
    """Rank 60 Gram matrix of 200 vectors (140 eigenvalues at roundoff)."""
    x = np.random.default_rng(5).standard_normal((60, 4000))
    m = np.random.default_rng(6).standard_normal((200, 60)) @ x
    g = m @ m.T
    check(g, *eigh(g))


def test_tridiagonal_and_diagonal_inputs():
    """Already tridiagonal (every reflector trivial) and diagonal inputs."""
    rng = np.random.default_rng(9)
    n = 70
    t = np.diag(rng.standard_normal(n)) + np.diag(rng.standard_normal(n - 1), 1)
    t = t + np.triu(t, 1).T
    check(t, *eigh(t))
    dg = np.diag(np.repeat([1.0, -2.0, 3.0, 0.5], 20)[:n])
    check(dg, *eigh(dg))


def test_pipeline_with_the_library_eigensolver(golden):
    """The whole path on the reference's small system with the library's
    eigensolver: the same Ritz values as with cuSOLVER and as the reference
    program's eval.dat."""
    g = golden("ref_small.npz")
    dims = tuple(int(v) for v in g["dims"])
    n = int(np.prod(dims))
    start = sep.start_states(int(g["run_seed"]), 4, n, float(g["dv"]))
    out = {}
    for mode in (0, 1):
        ctx = sep.Context(dims, (float(g["dx"]), float(g["dy"]), float(g["dz"])), potl=g["potl"])
        ctx.set_eigensolver(mode)
        out[mode] = ctx.pipeline(start, g["el"], 128, float(g["vmin"]))
        ctx.close()
    assert out[0]["mkept"] == out[1]["mkept"] == len(g["run_eval"])
    assert np.abs(out[1]["eval"] - g["run_eval"]).max() <= 1e-8
    assert np.abs(out[1]["eval"] - out[0]["eval"]).max() <= 1e-10
