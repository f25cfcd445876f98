"""Gradients of band-edge eigenvalues with respect to the form-factor
parameters (no counterpart in the reference, which fits its parameters with a
derivative-free Monte Carlo search, pseudopotFitting/fit.c:29-50).

Forward (C ABI): sep_potential_from_params (tables of pot.c:35-63, shifted as
filter/read.c:105-108, V(r) of filter/init.c:157-182 on the GPU), then
sep_pipeline (filter/main.c:64-142) for the Ritz pairs.
Backward (C ABI): sep_band_edge_backward -- Hellmann-Feynman density
dL/dV(r_g) = dv sum_k dL/dE_k psi_k(r_g)^2 and the V(r) backward on the GPU,
then the adjoints of the table shift and of the sine transform on the host.
Hellmann-Feynman holds for eigenpairs; the Ritz pairs used here are converged
to sigma << 1, so the error is of order sigma^2.

The torch.autograd.Function wraps the forward and backward; torch only
carries the parameters and the band-edge eigenvalues.
"""
import numpy as np

from . import binding


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


def window_targets(elmin, elmax, ms):
    """Filter targets of one window, filter/init.c:210-211."""
    if ms == 1:
        return np.array([elmin], dtype=np.float64)
    d = (elmax - elmin) / float(ms - 1)
    return np.array([elmin + float(j) * d for j in range(ms)], dtype=np.float64)


class BandEdgeProblem:
    """One nanocrystal, fixed start states and filter settings; maps the
    form-factor parameters (ntype x a0..a3, flattened) to band-edge
    eigenvalues: the n_vb highest converged Ritz values of a filter run on the
    valence-edge targets and the n_cb lowest of a run on the conduction-edge
    targets (one reference run each, same start states)."""

    def __init__(self, system, vb_targets, cb_targets, n_vb=3, n_cb=4, nc=None, seed=-314159,
                 precision="f64", sigma_max=1e-6):
        self.S = system
        self.targets = (np.asarray(vb_targets, dtype=np.float64),
                        np.asarray(cb_targets, dtype=np.float64))
        self.n_vb, self.n_cb = n_vb, n_cb
        self.nc = nc or system.nc
        self.sigma_max = sigma_max
        self.ctx = binding.Context(system.dims, system.steps, precision=precision)
        self.start = binding.start_states(seed, system.ns, system.ngrid, system.dv)
        self.types = system.types.astype(np.int32)
        self.ntype = int(self.types.max()) + 1
        self.bounds = None

    def _select(self, ev, sg, side):
        ok = np.where(sg < self.sigma_max)[0]
        ok = ok[np.argsort(ev[ok])]
        n = self.n_vb if side == 0 else self.n_cb
        if len(ok) < n:
            raise ValueError(f"only {len(ok)} Ritz values converged to sigma < {self.sigma_max}")
        return ok[-n:] if side == 0 else ok[:n]

    def forward(self, theta, indices=None, bounds=None):
        """Band-edge eigenvalues (valence then conduction); keeps what backward needs.

        bounds = (vmin, dE) fixes the filter's spectral bounds; None computes
        them from the new potential (energy range on the first run) and stores
        them in self.bounds."""
        th = np.asarray(theta, dtype=np.float64).reshape(self.ntype, 4)
        self.ctx.potential_from_params(self.S.xyz, self.types, th, self.S.vol_per_atom, self.S.mins)
        vmin, dE = (self.ctx.info()["vmin"], 0.0) if bounds is None else bounds
        sel, e, psi, sig, runs = [], [], [], [], []
        for side in (0, 1):
            res = self.ctx.pipeline(self.start, self.targets[side], self.nc, vmin, dE=dE,
                                    want_psi=True)
            dE = res["timing"]["dE"]
            ev, sg = res["eval"], res["sigma"]
            idx = self._select(ev, sg, side) if indices is None else indices[side]
            sel.append(idx)
            e.append(ev[idx])
            psi.append(res["psi"][idx])
            sig.append(sg[idx])
            runs.append((ev, sg))
        if bounds is None:
            self.bounds = (vmin, dE)
        self.saved = dict(theta=th.copy(), psi=np.concatenate(psi), indices=tuple(sel),
                          sigma=np.concatenate(sig), runs=runs)
        return np.concatenate(e)

    def backward(self, dL_dE):
        """dL/dtheta (flattened) from dL/dE of the last forward."""
        sv = self.saved
        g = self.ctx.band_edge_backward(self.S.xyz, self.types, sv["theta"], self.S.vol_per_atom,
                                        self.S.mins, sv["psi"], np.asarray(dL_dE, dtype=np.float64))
        return g.reshape(-1)


def torch_function():
    """torch.autograd.Function mapping theta (ntype*4,) float64 -> band-edge E (2 n_each,)."""
    import torch

    class BandEdgeEnergies(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, problem, bounds=None):
            e = problem.forward(theta.detach().cpu().numpy(), bounds=bounds)
            ctx.problem = problem
            return torch.from_numpy(e).to(theta.dtype)

        @staticmethod
        def backward(ctx, grad_e):
            g = ctx.problem.backward(grad_e.detach().cpu().numpy())
            return torch.from_numpy(g).to(grad_e.dtype), None, None

    return BandEdgeEnergies
