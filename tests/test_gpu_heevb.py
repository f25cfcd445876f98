"""The library's batched Hermitian solver of the lowest eigenpairs
(csrc/sep_heevb.cu: one CTA per matrix, Householder tridiagonalisation,
bisection, inverse iteration, back-transformation), which replaces one zheev
per k-point of the bulk fit (pseudopotFitting/diag.c:12-48, lowest bands
fit.c:86-88), against numpy's eigh (LAPACK).

Tolerances relative to the largest |eigenvalue| s: eigenvalues 1e-12 s,
residuals |A x - lambda x| <= 1e-11 s, orthonormality 1e-11, and for exactly
degenerate eigenvalues the projector onto the cluster's vectors 1e-9 from
LAPACK's.
"""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep

pytestmark = pytest.mark.gpu


def _random_hermitian(rng, n):
    x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return 0.5 * (x + x.conj().T)


def _with_spectrum(rng, lam):
    n = len(lam)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return (q * lam) @ q.conj().T


def _check(a, nw, w, v):
    ref_w, ref_v = np.linalg.eigh(a)
    s = np.abs(ref_w).max()
    assert np.abs(w - ref_w[:nw]).max() <= 1e-12 * s
    r = a @ v - v * w
    assert np.abs(r).max() <= 1e-11 * s
    g = v.conj().T @ v
    assert np.abs(g - np.eye(nw)).max() <= 1e-11
    # degenerate clusters: compare projectors
    i = 0
    while i < nw:
        j = i + 1
        while j < nw and ref_w[j] - ref_w[j - 1] <= 1e-9 * s:
            j += 1
        if j < len(ref_w) and ref_w[j] - ref_w[j - 1] <= 1e-9 * s:
            i = j  # cluster cut by nw: skip
            continue
        p_got = v[:, i:j] @ v[:, i:j].conj().T
        p_ref = ref_v[:, i:j] @ ref_v[:, i:j].conj().T
        assert np.abs(p_got - p_ref).max() <= 1e-9, (i, j)
        i = j


@pytest.mark.parametrize("n,nmat,nw", [(2, 3, 2), (33, 4, 10), (100, 5, 32), (200, 3, 64),
                                       (387, 6, 32), (512, 2, 24)])
def test_random_hermitian_lowest_eigenpairs(n, nmat, nw):
    rng = np.random.default_rng(n)
    a = np.stack([_random_hermitian(rng, n) for _ in range(nmat)])
    w, v = sep.hermitian_lowest(a, nw)
    for m in range(nmat):
        _check(a[m], nw, w[m], v[m])


def test_degenerate_spectra():
    """Clusters of exactly equal eigenvalues (as at high-symmetry k-points),
    one crossing the last wanted band."""
    rng = np.random.default_rng(11)
    n = 150
    lam = np.sort(rng.uniform(-3, 3, n))
    lam[3:6] = lam[3]          # triple
    lam[10:12] = lam[10]       # pair
    lam[20:26] = lam[20]       # six
    lam[30:34] = lam[30]       # crosses nw = 32
    lam = np.sort(lam)
    a = np.stack([_with_spectrum(rng, lam) for _ in range(3)])
    w, v = sep.hermitian_lowest(a, 32)
    for m in range(3):
        _check(a[m], 32, w[m], v[m])


def test_eigenvalues_only_and_diagonal_input():
    rng = np.random.default_rng(5)
    a = np.stack([_random_hermitian(rng, 80), np.diag(np.arange(80.0)[::-1]).astype(complex)])
    w, v = sep.hermitian_lowest(a, 16, vectors=False)
    assert v is None
    for m in range(2):
        ref = np.linalg.eigvalsh(a[m])[:16]
        assert np.abs(w[m] - ref).max() <= 1e-12 * np.abs(np.linalg.eigvalsh(a[m])).max()


def test_bad_arguments():
    with pytest.raises(sep.SepError):
        sep.hermitian_lowest(np.eye(600, dtype=complex), 4)
    with pytest.raises(sep.SepError):
        sep.hermitian_lowest(np.eye(10, dtype=complex), 11)
