"""Double-float arithmetic for the FP64-class work of the pipeline
(sep_ctx_set_arith): the H applies of Rayleigh-Ritz (filter/Hmat.c:11-86) and
of sigma (filter/energy.c:88-119), and the polish's Newton filter
(filter/filter.c:59-83), against the same pipeline in IEEE FP64.

Both runs share the complex64 filter, ortho and the eigensolves; only the
line passes of those H applies differ (about 48 against 53 significant bits,
an H apply within 2e-14 relative of FP64).  Tolerances: Ritz values 1e-11 Ha;
sigma 1e-9 Ha absolute (sigma is a norm of H psi - E psi, rounded at about
1e-14 of |H psi|)."""
import numpy as np
import pytest

import semi_empirical_pseudopotentials_gb300 as sep
from semi_empirical_pseudopotentials_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    S = systems.make_system("r1.0nm_48_dd", 1.0, 48, ms=4, ns=8, nc=512, seed=3,
                            elmin=-0.35, elmax=-0.15)
    start = sep.start_states(-4242, S.ns, S.ngrid, S.dv)
    return S, start


def _run(S, start, arith, polish):
    ctx = sep.Context(S.dims, S.steps, precision="mixed")
    ctx.set_arith(arith)
    ctx.set_polish(polish, 0.01)
    ctx.potential_from_params(S.xyz, S.types.astype(np.int32),
                              np.stack([S.params[0], S.params[1]]), S.vol_per_atom, S.mins)
    res = ctx.pipeline(start, S.el, S.nc, ctx.info()["vmin"])
    ctx.close()
    return res


@pytest.mark.parametrize("polish", [0, 64])
def test_double_float_pipeline_matches_fp64(case, polish):
    S, start = case
    a = _run(S, start, "dd", polish)
    b = _run(S, start, "f64", polish)
    assert a["mkept"] == b["mkept"] > 0
    assert np.abs(a["eval"] - b["eval"]).max() <= 1e-11, np.abs(a["eval"] - b["eval"]).max()
    assert np.abs(a["sigma"] - b["sigma"]).max() <= 1e-9, np.abs(a["sigma"] - b["sigma"]).max()
    if polish:
        assert a["timing"]["polish_s"] > 0.0


def test_arith_modes_and_defaults():
    ctx = sep.Context((32, 32, 32), (1.0, 1.0, 1.0), potl=np.zeros(32 ** 3), precision="mixed")
    ctx.set_arith("f64")
    ctx.set_arith("dd")
    with pytest.raises(KeyError):
        ctx.set_arith("fp32")
    ctx.close()


def test_double_float_filter_in_an_fp64_context():
    """An FP64 context with set_arith("dd") runs the Newton filter
    (filter/filter.c:59-83) in double-float: within 1e-12 relative of the
    FP64 filter over 70 Newton steps (each step's rounding about 2^-47
    against FP64's 2^-53)."""
    dims, steps = (36, 40, 48), (0.8, 0.75, 0.7)
    rng = np.random.default_rng(5)
    n = int(np.prod(dims))
    pot = -1.2 * np.exp(-rng.uniform(0.5, 1.5) * np.linspace(-2, 2, n) ** 2)
    dv = steps[0] * steps[1] * steps[2]
    ctx = sep.Context(dims, steps, potl=pot, precision="f64")
    vmin = float(pot.min())
    nc, dE = 70, 40.0
    ar, ai, zn = sep.coefficients([-1.0, -0.6, -0.2], nc, dE, vmin, (nc / (2.5 * dE)) ** 2)
    start = sep.start_states(-23, 5, n, dv)
    f64 = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.set_arith("dd")
    ddv = ctx.filter(start, ar, zn, 4.0 / dE, vmin)
    ctx.close()
    rel = np.abs(ddv - f64).max() / np.abs(f64).max()
    assert 0.0 < rel < 1e-12, rel
