"""Subspace contractions of ortho (filter/ortho.c:11-52) and Rayleigh-Ritz
(filter/Hmat.c:11-86) on the tcgen05 tensor cores by exact splitting, against
an extended-precision reference and against the FP64-pipe path.

Tolerance, elementwise: the splitting rounds each element to 2^-55 of its
row's largest magnitude, so |C - C_exact| <= 2^-52 (max|a_i| sum|b_j| +
sum|a_i| max|b_j|) + 4 2^-53 (|A| |B|^T): the bound of an FP64 product plus
the row-scaling term (both well below 2^-52 |a_i| |b_j| sqrt(k))."""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep

pytestmark = pytest.mark.gpu

TOL = 4 * 2.0 ** -53


def _ctx():
    return sep.Context((16, 16, 16), (1.0, 1.0, 1.0), potl=np.zeros(4096))


def _rows(rng, m, k, spread=4.0):
    a = rng.standard_normal((m, k)) * np.exp(rng.uniform(-spread, spread, (m, 1)))
    a[0, : k // 7 + 1] *= 1e5   # a row with a few very large entries
    if m > 1:
        a[1] = 0.0              # and an empty row
    return a


def _bound(A, B):
    aa, ab = np.abs(A), np.abs(B)
    split = 2.0 ** -52 * (np.outer(aa.max(1), ab.sum(1)) + np.outer(aa.sum(1), ab.max(1)))
    return TOL * (aa @ ab.T) + split + 1e-300


def _check(C, A, B):
    exact = A.astype(np.longdouble) @ B.astype(np.longdouble).T
    bound = _bound(A, B)
    err = np.abs(C - exact.astype(np.float64))
    assert np.all(err <= bound), float(np.max(err / bound))


@pytest.mark.parametrize("m,n,k", [(200, 200, 2000), (130, 70, 3000), (1, 1, 33), (129, 65, 31),
                                   (57, 57, 46656), (20, 9, 30000)])
def test_gram_and_cross_products(m, n, k):
    """Includes one-tile products with long K (split over every SM)."""
    rng = np.random.default_rng(m * 1000 + n)
    ctx = _ctx()
    A = _rows(rng, m, k)
    B = _rows(rng, n, k)
    C = ctx.subspace_gemm(A, B, alpha=0.37)
    _check(C, 0.37 * A, B)
    if m == n:
        G = ctx.subspace_gemm(A)
        _check(G, A, A)
        assert np.array_equal(G, G.T)


@pytest.mark.parametrize("m,k,w", [(300, 200, 1000), (64, 512, 1024), (5, 3, 70)])
def test_rotation(m, k, w):
    rng = np.random.default_rng(k)
    ctx = _ctx()
    W = rng.standard_normal((m, k))
    X = _rows(rng, k, w)
    out = ctx.subspace_rotate(W, X)
    _check(out, W, X.T)


def test_tensor_core_and_fp64_pipe_agree_at_subspace_sizes():
    """512 states x 300k points (split-K over many CTAs): both paths within
    the FP64 bound of each other."""
    rng = np.random.default_rng(5)
    ctx = _ctx()
    A = _rows(rng, 512, 300000)
    B = rng.standard_normal((200, 300000))
    tc, tcx = ctx.subspace_gemm(A), ctx.subspace_gemm(B, A)
    ctx.set_subspace("f64")
    f64, f64x = ctx.subspace_gemm(A), ctx.subspace_gemm(B, A)
    ctx.set_subspace("tc")
    assert np.all(np.abs(tc - f64) <= 2 * _bound(A, A))
    assert np.all(np.abs(tcx - f64x) <= 2 * _bound(B, A))


def test_repeatable_bit_for_bit_and_many_tiles_per_sm():
    """Integer accumulation makes the result independent of scheduling: the
    same products twice are bitwise equal.  A rotation with ~1000 output
    tiles runs several tiles per SM through the same shared-memory stages."""
    rng = np.random.default_rng(9)
    ctx = _ctx()
    A = _rows(rng, 160, 70000)
    G1, G2 = ctx.subspace_gemm(A), ctx.subspace_gemm(A)
    assert np.array_equal(G1, G2)
    W = rng.standard_normal((300, 160))
    X = _rows(rng, 160, 40000)
    R1, R2 = ctx.subspace_rotate(W, X), ctx.subspace_rotate(W, X)
    assert np.array_equal(R1, R2)
    ctx.set_subspace("f64")
    R64 = ctx.subspace_rotate(W, X)
    ctx.set_subspace("tc")
    assert np.all(np.abs(R1 - R64) <= 2 * _bound(W, X.T))
