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
