"""Adjoint of band-edge eigenvalues with respect to the form-factor
parameters (sep_potential_from_params + sep_pipeline forward,
sep_band_edge_backward), against central finite differences (h = 1e-5) of
the whole GPU path and against the reference-derived gradient: central
differences of the reference's own filter program on the same system
(tests/golden/adjoint_ref_fd.npz, made by tests/golden/make_adjoint_fixture.py).

System: the 0.6 nm CdSe-like sphere (29 atoms, 32^3 grid) with the fitted
zb_cdse form factors; valence-edge and conduction-edge filter windows of two
targets each, 16 start states, nc = 8192.  Band edges: the HOMO triplet and
the 1S_e + 1P_e conduction states, all with sigma < 1e-6."""
import os

import numpy as np
import pytest

from semi_empirical_pseudopotentials_gb300 import adjoint, systems

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "adjoint_ref_fd.npz")
H = 1e-5
REL = 1e-6  # gradient tolerance, relative to the largest entry


@pytest.fixture(scope="module")
def case():
    g = np.load(GOLD)
    S = systems.make_system("adjoint_0.6nm", float(g["radius_nm"]), int(g["n"]), ms=2,
                            ns=int(g["ns"]), nc=int(g["nc"]), seed=0)
    P = adjoint.BandEdgeProblem(S, adjoint.window_targets(*g["window_vb"], 2),
                                adjoint.window_targets(*g["window_cb"], 2), n_vb=int(g["n_vb"]),
                                n_cb=int(g["n_cb"]), seed=int(g["seed"]),
                                sigma_max=float(g["sigma_max"]))
    th0 = g["theta"].copy()
    e0 = P.forward(th0)
    sigma = P.saved["sigma"].copy()
    bounds = P.bounds
    J = np.stack([P.backward(np.eye(len(e0))[k]) for k in range(len(e0))])
    plus, minus = [], []
    for j in range(len(th0)):
        tp, tm = th0.copy(), th0.copy()
        tp[j] += H
        tm[j] -= H
        # each run selects its band edges by the same rule as the base run (the
        # kept count of ortho, and so the Ritz list, can change by one)
        plus.append(P.forward(tp, bounds=bounds))
        minus.append(P.forward(tm, bounds=bounds))
    return dict(g=g, P=P, th0=th0, e0=e0, sigma=sigma, J=J, plus=np.array(plus),
                minus=np.array(minus))


def test_band_edges_converged_and_equal_to_the_reference_program(case):
    assert case["sigma"].max() < 1e-6
    assert np.abs(case["e0"] - case["g"]["edges"]).max() < 1e-8


def test_hellmann_feynman_matches_central_differences(case):
    J = case["J"]
    Jfd = (case["plus"] - case["minus"]).T / (2 * H)
    err = np.abs(J - Jfd).max()
    assert err <= REL * np.abs(J).max(), (err, np.abs(J).max())


def test_hellmann_feynman_matches_the_reference_derived_gradient(case):
    J, Jref = case["J"], case["g"]["jac_fd"]
    err = np.abs(J - Jref).max()
    assert err <= REL * np.abs(J).max(), (err, np.abs(J).max())


def test_loss_gradient_through_torch_autograd(case):
    torch = pytest.importorskip("torch")
    P, th0, e0 = case["P"], case["th0"], case["e0"]
    e_t = e0 + 0.01 * np.random.default_rng(21).uniform(-1, 1, e0.shape)  # seeded targets
    fn = adjoint.torch_function()
    theta = torch.tensor(th0, dtype=torch.float64, requires_grad=True)
    e = fn.apply(theta, P, P.bounds)
    loss = torch.sum((e - torch.from_numpy(e_t)) ** 2)
    loss.backward()
    g = theta.grad.numpy()

    def L(e):
        return np.sum((e - e_t) ** 2, axis=-1)

    gfd = (L(case["plus"]) - L(case["minus"])) / (2 * H)
    assert np.abs(g - gfd).max() <= REL * np.abs(g).max(), (g, gfd)
