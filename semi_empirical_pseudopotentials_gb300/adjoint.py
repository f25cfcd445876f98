"""Gradients of band-edge eigenvalues with respect to the form-factor
parameters (no counterpart in the reference, which fits its parameters with a
derivative-free Monte Carlo search, pseudopotFitting/fit.c:29-50).

Forward chain (each step is the reference's own):
  a0..a3 per species --pot.c:35-63--> real-space table v(r_k)
  --read.c:105-108--> table minus its last value
  --init.c:157-182--> V(r_g) on the grid (GPU, sep_vbuild)
  --main.c:64-142--> Ritz pairs (E_k, psi_k) of the filter path (GPU, sep_pipeline)
Backward chain:
  dL/dE_k --Hellmann-Feynman--> dL/dV(r_g) = sum_k dL/dE_k psi_k(r_g)^2 dv (GPU)
  --V(r) backward (GPU)--> dL/dtable --shift--> dL/draw table
  --analytic Jacobian of the sine transform--> dL/da.
Hellmann-Feynman holds for eigenpairs; the Ritz pairs used here are
converged to sigma << 1 so the error is of order sigma^2.

The torch.autograd.Function wraps the forward and backward; torch only
carries the 8 parameters and the 8 eigenvalues.
"""
import numpy as np

from . import binding

NG = 1024
PI = 3.14159265358979323846
TWO_PI = 6.28318530717958647692


def _q_grid():
    """q_i = i dq by running sums from 0, as pot.c:39."""
    dq = (5.0 - 0.0) / NG
    q = np.empty(NG)
    s = 0.0
    for i in range(NG):
        q[i] = s
        s += dq
    return q, dq


def form_factor_jacobian(params, vol_per_atom):
    """Table v(r_k) (pot.c:35-63, from the library) and dv/da_j [4, 1024].

    v = S vq with S[k][i] = C_k q_i sin(q_i r_k), S[0][i] = C_0 q_i^2 and
    vq_i = f(q_i) vol; f(q) = a0 (q^2 - a1)/(a2 e^{a3 q^2} + 1)
    (pseudopotFitting/hamiltonian.c:91-94).
    """
    a = np.asarray(params, dtype=np.float64)
    r, v = binding.form_factor_table(a, vol_per_atom)
    q, dq = _q_grid()
    q2 = q * q
    E = np.exp(a[3] * q2)
    D = a[2] * E + 1.0
    num = q2 - a[1]
    dfa = np.stack([num / D, -a[0] / D, -a[0] * num * E / D ** 2,
                    -a[0] * num * a[2] * q2 * E / D ** 2]) * vol_per_atom  # [4, NG]
    S = np.empty((NG, NG))
    pref = TWO_PI ** 3
    S[1:] = (dq * 4.0 * PI / (pref * r[1:]))[:, None] * q[None, :] * np.sin(np.outer(r[1:], q))
    S[0] = (dq * 4.0 * PI / pref) * q2
    return r, v, dfa @ S.T  # [4, NG]


def shift_backward(d_shifted, n):
    """Adjoint of v_i <- v_i - v_{n-1} (filter/read.c:105-108)."""
    d = np.array(d_shifted, dtype=np.float64, copy=True)
    d[n - 1] = -np.sum(d_shifted[:n - 1])
    return d


def select_band_edges(ev, sigma, n_each=4, sigma_max=1e-5, window=None):
    """Indices of the n_each highest valence and n_each lowest conduction Ritz
    values: the gap is the widest spacing among converged values in `window`."""
    ok = np.where(sigma < sigma_max)[0]
    if window is not None:
        ok = ok[(ev[ok] >= window[0]) & (ev[ok] <= window[1])]
    ok = ok[np.argsort(ev[ok])]
    if len(ok) < 2 * n_each:
        raise ValueError(f"only {len(ok)} converged Ritz values in the window")
    e = ev[ok]
    lo, hi = n_each - 1, len(ok) - n_each  # gap between positions g and g+1
    g = lo + int(np.argmax(np.diff(e)[lo:hi]))
    return np.concatenate([ok[g - n_each + 1:g + 1], ok[g + 1:g + 1 + n_each]])


class BandEdgeProblem:
    """One nanocrystal, fixed start states and filter settings; maps the
    8 form-factor parameters (2 species x a0..a3) to band-edge eigenvalues."""

    def __init__(self, system, nc=None, seed=-314159, precision="f64", sigma_max=1e-5,
                 n_each=4, window=None):
        self.S = system
        self.nc = nc or system.nc
        self.sigma_max = sigma_max
        self.n_each = n_each
        self.window = window
        self.ctx = binding.Context(system.dims, system.steps, precision=precision)
        self.start = binding.start_states(seed, system.ns, system.ngrid, system.dv)
        self.types = system.types.astype(np.int32)
        self.species = sorted(int(t) for t in np.unique(system.types))

    def tables(self, theta):
        theta = np.asarray(theta, dtype=np.float64).reshape(len(self.species), 4)
        ntype = max(self.species) + 1
        tr = np.zeros((ntype, NG))
        tv = np.zeros((ntype, NG))
        jac = {}
        for k, t in enumerate(self.species):
            r, v, dv = form_factor_jacobian(theta[k], self.S.vol_per_atom)
            tr[t] = r
            tv[t] = v - v[-1]
            jac[t] = dv
        return tr, tv, jac

    def forward(self, theta, indices=None):
        """Band-edge eigenvalues; also keeps what backward needs."""
        tr, tv, jac = self.tables(theta)
        ntype = tr.shape[0]
        tab_n = np.full(ntype, NG, dtype=np.int64)
        self.ctx.vbuild(self.S.xyz, self.types, tr, tv, tab_n, self.S.mins, install=True)
        vmin = self.ctx.info()["vmin"]
        res = self.ctx.pipeline(self.start, self.S.el, self.nc, vmin, want_psi=True)
        ev, sg = res["eval"], res["sigma"]
        if indices is None:
            indices = select_band_edges(ev, sg, self.n_each, self.sigma_max, self.window)
        self.saved = dict(tr=tr, tv=tv, jac=jac, tab_n=tab_n, psi=res["psi"][indices],
                          indices=indices, sigma=sg[indices])
        return ev[indices].copy()

    def backward(self, dL_dE):
        """dL/dtheta from dL/dE of the last forward."""
        sv = self.saved
        rho = self.ctx.hf_density(sv["psi"], np.asarray(dL_dE, dtype=np.float64))
        dtab, _ = self.ctx.vbuild_backward(self.S.xyz, self.types, sv["tr"], sv["tv"],
                                           sv["tab_n"], self.S.mins, rho)
        grads = []
        for t in self.species:
            d_raw = shift_backward(dtab[t], NG)
            grads.append(sv["jac"][t] @ d_raw)
        return np.concatenate(grads)


def torch_function():
    """torch.autograd.Function mapping theta (8,) float64 -> band-edge E (2 n_each,)."""
    import torch

    class BandEdgeEnergies(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, problem):
            e = problem.forward(theta.detach().cpu().numpy())
            ctx.problem = problem
            return torch.from_numpy(e).to(theta.dtype)

        @staticmethod
        def backward(ctx, grad_e):
            g = ctx.problem.backward(grad_e.detach().cpu().numpy())
            return torch.from_numpy(g).to(grad_e.dtype), None

    return BandEdgeEnergies
