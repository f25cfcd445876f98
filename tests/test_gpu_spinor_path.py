"""The spinor filter program on the GPU (sep_spinor_*, through the C ABI):
the spinor Hamiltonian, the Newton filter with complex coefficients, the
energy range and the whole program against the reference's own routines
(tests/golden/spinor_vso.npz, made by tests/golden/make_spinor_fixture.py
from spinors/filterSpinors/*.c) and against the oracle on a larger case.

Tolerances: H psi and the filter output as the CPU oracle's pins (samples
to 1e-12 of the largest, row sums and sums of squares to 1e-11); Vmin and
dE to 1e-9; the kept count exactly; Ritz values to 1e-9 (relative) and
sigma to 1e-7 (relative)."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import spinor_oracle as so
from semi_empirical_pseudopotentials_gb300 import binding, spinor

pytestmark = pytest.mark.gpu

EKINMAX = 20.0  # filterSpinors/init.c:23


def load(golden):
    g = golden("spinor_vso.npz")
    raw = g["nlc"]
    return g, raw.reshape(-1).view(so.NLC_DTYPE).reshape(raw.shape[:2])


def check_sampled(g, name, got):
    got = np.asarray(got).reshape(-1, 2 * int(np.prod(g["dims"])))
    ref = g[name + "_sample"].reshape(got.shape[0], -1)
    scale = np.abs(ref).max()
    assert np.abs(got[:, g["sample_idx"]] - ref).max() <= 1e-12 * scale
    assert np.allclose(got.sum(axis=1), g[name + "_sum"], rtol=1e-11, atol=1e-12 * scale)
    assert np.allclose((np.abs(got) ** 2).sum(axis=1), g[name + "_sumsq"], rtol=1e-11, atol=0)


def path(g, nlc, form="gauss"):
    dims = tuple(int(v) for v in g["dims"])
    h = float(g["h"])
    ctx = binding.Context(dims, (h, h, h), potl=g["potl"], ekinmax=EKINMAX)
    assert np.array_equal(ctx_ksqr(ctx), g["ksqr"])
    if form == "gauss":
        return ctx, spinor.SpinorPath(ctx, nlc, g["nl"], sigma=h)
    return ctx, spinor.SpinorPath(ctx, nlc, g["nl"], elkb=g["elkb"])


def ctx_ksqr(ctx):
    import ctypes as C

    out = np.empty(ctx.ngrid)
    L = binding.lib()
    L.sep_ctx_ksqr.argtypes = [C.c_void_p, C.c_void_p]
    binding._check(L.sep_ctx_ksqr(ctx.h, out.ctypes.data))
    return out


@pytest.mark.parametrize("form", ["gauss", "kb"])
def test_spinor_hamiltonian_matches_reference(golden, form):
    g, nlc = load(golden)
    ctx, sp = path(g, nlc, form)
    check_sampled(g, "h_" + form, sp.hamiltonian(g["psi"]))


def test_spinor_newton_filter_matches_reference(golden):
    g, nlc = load(golden)
    ctx, sp = path(g, nlc)
    got = sp.filter(g["psi"][None, :], g["an"], g["zn"], float(g["dE_1"]), float(g["vmin"]))
    check_sampled(g, "filter_out", got[0])


def test_spinor_energy_range_matches_reference(golden):
    g, nlc = load(golden)
    ctx, sp = path(g, nlc)
    vmin, dE, _ = sp.energy_range()
    assert abs(vmin - float(g["run_vmin"])) <= 1e-9 * abs(float(g["run_vmin"]))
    assert abs(dE - float(g["run_dE"])) <= 1e-9 * float(g["run_dE"])


def test_spinor_pipeline_matches_reference_program(golden):
    """The reference's whole spinor program (energy range, coefficients,
    start spinors from its seed, filtering, portho, Hmat, sigma)."""
    g, nlc = load(golden)
    ctx, sp = path(g, nlc)
    n = ctx.ngrid
    ns = int(g["run_ns"])
    st = O.start_states(int(g["run_seed"]), 2 * ns, n, ctx.dv)
    spinors = np.stack([np.concatenate([st[2 * j], st[2 * j + 1]]) for j in range(ns)])
    res = sp.pipeline(spinors.astype(np.complex128), g["run_el"], int(g["run_nc"]))
    assert res["mkept"] == int(g["run_mkept"])
    assert abs(res["timing"]["dE"] - float(g["run_dE"])) <= 1e-9 * float(g["run_dE"])
    assert np.allclose(res["eval"], g["run_eval"], rtol=1e-9, atol=1e-12)
    assert np.allclose(res["sigma"], g["run_sigma"], rtol=1e-7, atol=1e-10)


def larger_case(seed=11, n=32, h=0.6, natom=12):
    rng = np.random.default_rng(seed)
    v = -0.5 * n * h + h * np.arange(n)
    rxyz = rng.uniform(-5.0, 5.0, size=(natom, 3))
    nlc, nl = so.neighbour_lists(v, v, v, rxyz, rng.uniform(-0.15, 0.15, natom),
                                 0.49 * 6.0 * np.log(10.0), 1200)
    zz, yy, xx = np.meshgrid(v, v, v, indexing="ij")
    pot = np.zeros(n ** 3)
    for a in range(natom):
        d2 = (xx - rxyz[a, 0]) ** 2 + (yy - rxyz[a, 1]) ** 2 + (zz - rxyz[a, 2]) ** 2
        pot -= 0.5 * np.exp(-0.4 * d2).ravel()
    return (n, n, n), h, nlc, nl, pot


def test_spinor_filter_against_oracle_on_a_larger_case():
    """32^3 grid, 12 atoms, 3 start spinors x 3 complex targets over 40
    Newton steps against the oracle's newton_filter."""
    dims, h, nlc, nl, pot = larger_case()
    ctx = binding.Context(dims, (h, h, h), potl=pot, ekinmax=EKINMAX)
    sp = spinor.SpinorPath(ctx, nlc, nl, sigma=h)
    n = ctx.ngrid
    rng = np.random.default_rng(4)
    start = rng.normal(size=(3, 2 * n)) + 1j * rng.normal(size=(3, 2 * n))
    nc = 40
    an = rng.normal(size=(3, nc)) + 1j * rng.normal(size=(3, nc))
    an /= np.arange(1, nc + 1) ** 2
    zn = rng.uniform(-2.0, 2.0, nc)
    dE_1, vmin = 4.0 / 30.0, float(pot.min())
    got = sp.filter(start, an, zn, dE_1, vmin)
    ks = ctx_ksqr(ctx)
    for s in range(3):
        ref = so.newton_filter(start[s], an, zn, dE_1, vmin, pot, ks, dims, nlc, nl, h, h ** 3)
        assert np.abs(got[s] - ref).max() <= 1e-11 * np.abs(ref).max(), s


def test_spinor_pipeline_library_eigensolver_matches_cusolver():
    """The whole spinor program on the 32^3 case with the library's solver
    (on the real embedding of each Hermitian problem) and with cuSOLVER's
    Zheevd: the same kept count, Ritz values to 1e-10 and sigma to 1e-8."""
    dims, h, nlc, nl, pot = larger_case()
    out = {}
    for mode in (1, 0):
        ctx = binding.Context(dims, (h, h, h), potl=pot, ekinmax=EKINMAX)
        ctx.set_eigensolver(mode)
        sp = spinor.SpinorPath(ctx, nlc, nl, sigma=h)
        n = ctx.ngrid
        st = O.start_states(-4242, 8, n, ctx.dv)
        spinors = np.stack([np.concatenate([st[2 * j], st[2 * j + 1]]) for j in range(4)])
        out[mode] = sp.pipeline(spinors.astype(np.complex128), [-0.8, -0.6, -0.4], 64)
        ctx.close()
    assert out[0]["mkept"] == out[1]["mkept"]
    assert np.abs(out[0]["eval"] - out[1]["eval"]).max() <= 1e-10
    assert np.abs(out[0]["sigma"] - out[1]["sigma"]).max() <= 1e-8
