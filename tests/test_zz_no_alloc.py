"""sep_normalize_states_noalloc (fixed device scratch, no allocation) against
sep_normalize_states (host arrays, allocates per call) on the same states.

Both run the same two-level reduction and scaling kernels with the same launch
shapes, so the results agree to rounding; the tolerance below is 1e-14
relative.  Collected last so that it also runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep

pytestmark = pytest.mark.gpu

RTOL = 1e-14


def _lib():
    L = sep.lib()
    L.sep_normalize_states.argtypes = [C.POINTER(C.c_double), C.c_long, C.c_long, C.c_double]
    L.sep_normalize_states_noalloc.argtypes = [C.c_void_p, C.c_long, C.c_long, C.c_double,
                                               C.c_void_p]
    return L


def _reference(L, psi, dv):
    out = np.ascontiguousarray(psi, dtype=np.float64).copy()
    m, n = out.shape
    st = L.sep_normalize_states(out.ctypes.data_as(C.POINTER(C.c_double)), m, n, dv)
    assert st == 0, L.sep_last_error()
    return out


def _noalloc(L, torch, psi, dv):
    d = torch.from_numpy(np.ascontiguousarray(psi, dtype=np.float64)).to("cuda:0")
    stream = torch.cuda.current_stream(0)
    m, n = psi.shape
    st = L.sep_normalize_states_noalloc(C.c_void_p(d.data_ptr()), m, n, dv,
                                        C.c_void_p(stream.cuda_stream))
    assert st == 0, L.sep_last_error()
    stream.synchronize()
    return d.cpu().numpy()


def test_noalloc_normalize_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = _lib()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(2024)
    cases = [(7, 32 * 36 * 40, 0.3), (1024, 4096, 0.125)]  # odd count; the row limit
    for m, n, dv in cases:  # two calls in a row, the second on the largest block
        psi = rng.standard_normal((m, n)) * rng.uniform(0.1, 10.0, (m, 1))
        ref = _reference(L, psi, dv)
        got = _noalloc(L, torch, psi, dv)
        assert np.allclose(got, ref, rtol=RTOL, atol=0.0), np.abs(got - ref).max()
        assert np.allclose(np.sum(got * got, axis=1) * dv, 1.0, rtol=1e-12, atol=0.0)


def test_noalloc_back_to_back_calls_without_synchronising():
    """Several calls of different sizes queued on one stream, then on the NULL
    (legacy default) stream, with one synchronise at the end of each run: the
    shared scratch is reused by each call after the previous one finished on
    the stream, and every block matches the allocating entry point."""
    torch = pytest.importorskip("torch")
    L = _lib()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(77)
    shapes = [(1024, 2048), (3, 50000), (1, 17), (513, 4096), (64, 36 * 36 * 36)]
    blocks = [rng.standard_normal(s) * rng.uniform(0.5, 4.0, (s[0], 1)) for s in shapes]
    dv = 0.42
    refs = [_reference(L, b, dv) for b in blocks]
    for stream in (torch.cuda.Stream(0), None):
        devs = [torch.from_numpy(b).to("cuda:0") for b in blocks]
        torch.cuda.synchronize()
        handle = None if stream is None else C.c_void_p(stream.cuda_stream)
        for d in devs:
            m, n = d.shape
            st = L.sep_normalize_states_noalloc(C.c_void_p(d.data_ptr()), m, n, dv, handle)
            assert st == 0, L.sep_last_error()
        torch.cuda.synchronize()
        for d, ref in zip(devs, refs):
            got = d.cpu().numpy()
            assert np.allclose(got, ref, rtol=RTOL, atol=0.0), np.abs(got - ref).max()


def test_noalloc_rejects_more_states_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    L = _lib()
    d = torch.zeros((1025, 16), dtype=torch.float64, device="cuda:0")
    st = L.sep_normalize_states_noalloc(C.c_void_p(d.data_ptr()), 1025, 16, 1.0, None)
    assert st == -1
    assert b"1024" in L.sep_last_error()
