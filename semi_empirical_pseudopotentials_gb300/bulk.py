"""Bulk band structures for the empirical-pseudopotential fit (the
reference's pseudopotFitting/ program), on the GPU, with gradients.

* ``read_fit_inputs(directory)`` reads the reference's inputs (input.par,
  multiInput.par, system_<i>.par, kpoints_<i>.par, expBandStruct_<i>.par and
  <Symbol>Params.par; read.c:8-171, init.c:60-93).
* ``BulkCrystal`` holds one crystal on the GPU (sep_bulk_create) and returns
  its band structure in eV (sep_bulk_bands: fit.c:71-97) or the
  Hellmann-Feynman gradient of a loss of it (sep_bulk_bands_backward).
* ``BulkFit`` is the reference's fit objective, the band-weighted mean
  squared error averaged over the band structures (fit.c:101-145), with its
  gradient in the fit parameters: 4 form-factor parameters per distinct
  element, shared by every crystal, a0 scaled by the ratio of volumes per
  atom between crystals (fit.c:193-245).  The reference searches these by
  Monte Carlo (fit.c:9-69); the gradient lets any optimiser do it.
* ``BandStructureMSE`` wraps the objective as a torch.autograd.Function.
* ``write_band_structure`` writes bandStruct_<i>.dat ("% .5f " columns,
  write.c:54-66).

The band structures are computed by libsep_gb300.so; only the scalar loss and
the chain from crystal parameters to fit parameters are host arithmetic.
"""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from .binding import SepError, _check, lib

TWOPI = 6.28318530717958647692

_INPUT_FIELDS = {"maxKE": float, "nBandStructures": int, "nAtoms": int, "nElectrons": int,
                 "nIterations": int, "nKPoints": int, "beta": float, "stepSize": float,
                 "kineticEnergyScaling": float, "scale": float}


@dataclass
class Crystal:
    """One band structure's system (read.c:103-171), lengths in bohr."""
    cell: np.ndarray            # 3 x 3 rows a0, a1, a2 (scaled)
    symbols: list
    tau: np.ndarray             # natom x 3
    kpts: np.ndarray            # nk x 3, times 2 pi / scale
    max_ke: float
    ne: int
    scale: float
    exp_bands: np.ndarray | None = None   # nk x ne (eV)
    volume: float = 0.0
    vol_per_atom: float = 0.0
    atom_params: np.ndarray | None = None  # natom x 4 as the reference initialises them


@dataclass
class FitInputs:
    crystals: list
    elements: list              # distinct symbols, first appearance first
    params: np.ndarray          # len(elements) x 4 (from <Symbol>Params.par)
    norm_vol: list = field(default_factory=list)   # normalizedVolPerAtom per crystal
    ke_scale: float = 1.0
    beta: float = 0.0
    step_size: float = 0.0
    n_iterations: int = 0


def _pairs(text, path):
    tok = text.split()
    out = {}
    i = 0
    while i < len(tok):
        name = tok[i]
        if name not in _INPUT_FIELDS or i + 2 >= len(tok) or tok[i + 1] != "=":
            raise ValueError(f"{path}: Invalid input field and/ or format of input ({name})")
        out[name] = _INPUT_FIELDS[name](tok[i + 2])
        i += 3
    return out


def _floats(path):
    with open(path) as f:
        return [float(t) for t in f.read().split()]


def _read_system(path, na):
    """system_<i>.par: "scale = s", "cell" + 3 rows, "atoms" + na lines
    (read.c:126-152)."""
    with open(path) as f:
        tok = f.read().split()
    scale, cell, symbols, pos = None, None, [], []
    i = 0
    while i < len(tok):
        if tok[i] == "atoms":
            for a in range(na):
                symbols.append(tok[i + 1 + 4 * a])
                pos.append([float(t) for t in tok[i + 2 + 4 * a:i + 5 + 4 * a]])
            i += 1 + 4 * na
        elif tok[i] == "cell":
            cell = np.array([float(t) for t in tok[i + 1:i + 10]]).reshape(3, 3)
            i += 10
        elif tok[i] == "scale":
            scale = float(tok[i + 2])
            i += 3
        else:
            i += 1
    if cell is None or len(symbols) != na:
        raise ValueError(f"{path}: needs a cell and {na} atoms")
    return scale, cell, symbols, np.array(pos, dtype=np.float64)


def _cell_volume(cell):
    a = cell
    c = np.array([a[1][1] * a[2][2] - a[1][2] * a[2][1], a[1][2] * a[2][0] - a[1][0] * a[2][2],
                  a[1][0] * a[2][1] - a[1][1] * a[2][0]])
    return float(a[0][0] * c[0] + a[0][1] * c[1] + a[0][2] * c[2])


def read_fit_inputs(directory) -> FitInputs:
    """The reference's fit inputs in ``directory`` (read.c:8-171, init.c:60-93).
    A scale given in input.par (older runs) applies when system_<i>.par has
    none."""
    d = str(directory)
    with open(os.path.join(d, "input.par")) as f:
        inp = _pairs(f.read(), os.path.join(d, "input.par"))
    nbs = int(inp.get("nBandStructures", 1))
    if nbs > 1:                                           # read.c:59-78
        with open(os.path.join(d, "multiInput.par")) as f:
            tok = f.read().split()
        per = []
        for i in range(nbs):
            grp = _pairs(" ".join(tok[12 * i:12 * i + 12]), "multiInput.par")
            per.append((grp["nAtoms"], grp["nElectrons"], grp["nKPoints"], grp["maxKE"]))
    else:                                                 # read.c:47-56
        per = [(inp["nAtoms"], inp["nElectrons"], inp["nKPoints"], inp["maxKE"])]
    crystals = []
    for i, (na, ne, nk, mke) in enumerate(per):
        scale, cell, symbols, pos = _read_system(os.path.join(d, f"system_{i}.par"), na)
        if scale is None:
            scale = inp.get("scale")
        if scale is None:
            raise ValueError(f"system_{i}.par: no scale")
        cell = cell * scale                               # read.c:154-157
        colsum = cell[0] + cell[1] + cell[2]
        tau = pos * colsum                                # read.c:160-165
        k = np.array(_floats(os.path.join(d, f"kpoints_{i}.par"))[:3 * nk]).reshape(nk, 3)
        k = k * (TWOPI / scale)                           # read.c:115-118
        exp = None
        ep = os.path.join(d, f"expBandStruct_{i}.par")
        if os.path.exists(ep):
            vals = _floats(ep)[:nk * (ne + 1)]
            exp = np.array(vals).reshape(nk, ne + 1)[:, 1:]
        vol = _cell_volume(cell)
        crystals.append(Crystal(cell=cell, symbols=symbols, tau=tau, kpts=k, max_ke=float(mke),
                                ne=int(ne), scale=float(scale), exp_bands=exp, volume=vol,
                                vol_per_atom=vol / na))
    norm_vol = [crystals[0].vol_per_atom / c.vol_per_atom for c in crystals]   # read.c:170
    elements, params, src = [], [], {}
    for ci, c in enumerate(crystals):
        for s in c.symbols:
            if s not in src:
                src[s] = ci
                elements.append(s)
                params.append(_floats(os.path.join(d, f"{s}Params.par"))[:4])
    fit = FitInputs(crystals=crystals, elements=elements, params=np.array(params),
                    norm_vol=norm_vol, ke_scale=float(inp.get("kineticEnergyScaling", 1.0)),
                    beta=float(inp.get("beta", 0.0)), step_size=float(inp.get("stepSize", 0.0)),
                    n_iterations=int(inp.get("nIterations", 0)))
    for ci, c in enumerate(crystals):
        c.atom_params = np.array([fit_atom_params(fit, fit.params, ci, s) for s in c.symbols])
    return fit


def fit_atom_params(fit, theta, ci, symbol):
    """An atom's parameters in crystal ci: its element's, with a0 scaled by
    normalizedVolPerAtom[ci] / normalizedVolPerAtom[first crystal of the
    element] (init.c:72-80, fit.c:203-207)."""
    e = fit.elements.index(symbol)
    first = next(i for i, c in enumerate(fit.crystals) if symbol in c.symbols)
    p = np.array(theta[e], dtype=np.float64)
    if first != ci:
        p[0] *= fit.norm_vol[ci] / fit.norm_vol[first]
    return p


def basis(cell, max_ke):
    """Plane waves with |G|^2/2 < max_ke (sep_bulk_basis), nbv x 3."""
    L = lib()
    cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
    dp = C.POINTER(C.c_double)
    n = C.c_long()
    _check(L.sep_bulk_basis(cell.ctypes.data_as(dp), float(max_ke), 0, C.byref(n), None))
    g = np.zeros((n.value, 3))
    _check(L.sep_bulk_basis(cell.ctypes.data_as(dp), float(max_ke), n.value, C.byref(n),
                            g.ctypes.data_as(dp)))
    return g


class BulkCrystal:
    """One crystal's band structure on the GPU (sep_bulk_*)."""

    def __init__(self, crystal: Crystal, ke_scale=1.0, nev=None):
        self.crystal = crystal
        self.types_of = []
        for s in crystal.symbols:
            if s not in self.types_of:
                self.types_of.append(s)
        types = np.array([self.types_of.index(s) for s in crystal.symbols], dtype=np.int32)
        self.g = basis(crystal.cell, crystal.max_ke)
        self.nbv = len(self.g)
        self.nk = len(crystal.kpts)
        self.nev = int(nev or crystal.ne)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        tau = np.ascontiguousarray(crystal.tau, dtype=np.float64)
        kp = np.ascontiguousarray(crystal.kpts, dtype=np.float64)
        self._h = C.c_void_p()
        _check(lib().sep_bulk_create(self.nbv, self.g.ctypes.data_as(dp), len(tau),
                                     tau.ctypes.data_as(dp), types.ctypes.data_as(ip),
                                     len(self.types_of), self.nk, kp.ctypes.data_as(dp),
                                     float(ke_scale), self.nev, C.byref(self._h)))

    def type_params(self, atom_params):
        """ntype x 4 from per-atom parameters (the first atom of each type)."""
        ap = np.asarray(atom_params, dtype=np.float64)
        return np.ascontiguousarray([ap[self.crystal.symbols.index(s)] for s in self.types_of])

    def bands(self, type_params, keep_vectors=False):
        """nk x nev bands in eV.  keep_vectors: also keep the eigenvectors, so
        that backward() with the same parameters needs no second solve."""
        p = np.ascontiguousarray(type_params, dtype=np.float64).reshape(-1, 4)
        out = np.zeros((self.nk, self.nev))
        dp = C.POINTER(C.c_double)
        f = lib().sep_bulk_bands_keep if keep_vectors else lib().sep_bulk_bands
        _check(f(self._h, p.ctypes.data_as(dp), out.ctypes.data_as(dp)))
        return out

    def backward(self, type_params, dl_de):
        """(bands, dL/dparams ntype x 4) for dL/dE (nk x nev, per eV)."""
        p = np.ascontiguousarray(type_params, dtype=np.float64).reshape(-1, 4)
        g = np.ascontiguousarray(dl_de, dtype=np.float64).reshape(self.nk, self.nev)
        out = np.zeros((self.nk, self.nev))
        grad = np.zeros_like(p)
        dp = C.POINTER(C.c_double)
        _check(lib().sep_bulk_bands_backward(self._h, p.ctypes.data_as(dp), g.ctypes.data_as(dp),
                                             out.ctypes.data_as(dp), grad.ctypes.data_as(dp)))
        return out, grad

    def set_solver(self, batched):
        """cuSOLVER: True its batched eigensolver (default), False one matrix per call."""
        _check(lib().sep_bulk_set_solver(self._h, 1 if batched else 0))

    def set_eigensolver(self, mode):
        """"native" (default): the library's batched solver of the lowest bands;
        "cusolver": cuSOLVER (see set_solver)."""
        if mode not in ("native", "cusolver"):
            raise ValueError("eigensolver: 'native' or 'cusolver'")
        _check(lib().sep_bulk_set_eigensolver(self._h, 1 if mode == "native" else 0))

    @property
    def solver_path(self):
        v = C.c_int()
        _check(lib().sep_bulk_solver_path(self._h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sep_bulk_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def band_weights(ne):
    """fit.c:106-112: band-edge bands weigh 4, the next 2, the deepest 0.06125."""
    w = np.zeros(ne)
    for j in range(ne // 2):
        val = 0.06125 if j < ne // 8 else (2.0 if j < ne // 4 else 4.0)
        w[j] = w[ne - j - 1] = val
    return w


class BulkFit:
    """The reference's fit objective on the GPU, with its gradient."""

    def __init__(self, fit: FitInputs):
        self.fit = fit
        self.crystals = [BulkCrystal(c, fit.ke_scale) for c in fit.crystals]

    def crystal_params(self, theta):
        out = []
        for ci, bc in enumerate(self.crystals):
            out.append(np.array([fit_atom_params(self.fit, theta, ci, s) for s in bc.types_of]))
        return out

    def _each_crystal(self, fn, theta):
        """fn(ci, crystal, params) for every crystal at once: each crystal has
        its own stream, and the library calls release the GIL, so the
        crystals' solves share the GPU."""
        jobs = list(zip(range(len(self.crystals)), self.crystals, self.crystal_params(theta)))
        if len(jobs) == 1:
            return [fn(*jobs[0])]
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            return list(ex.map(lambda j: fn(*j), jobs))

    def band_structures(self, theta):
        return self._each_crystal(lambda ci, bc, p: bc.bands(p), theta)

    def _mse_terms(self, ci, b, weighted=True):
        exp = self.fit.crystals[ci].exp_bands
        w = np.broadcast_to(band_weights(b.shape[1]) if weighted else np.ones(b.shape[1]),
                            b.shape)
        use = np.abs(exp) > 1e-10                         # fit.c:133-138
        n = np.count_nonzero(use)
        r = np.where(use, b - exp, 0.0)
        return float(np.sum(w * r * r) / n), 2.0 * w * r / n

    def objective(self, theta, weighted=True):
        """calcAllIndividualWeightedMSE (fit.c:101-122), or with weighted=False
        calcAllIndividualMSE (fit.c:147-177)."""
        bs = self.band_structures(theta)
        return sum(self._mse_terms(i, b, weighted)[0] for i, b in enumerate(bs)) / len(bs)

    def objective_and_grad(self, theta):
        theta = np.asarray(theta, dtype=np.float64)
        nbs = len(self.crystals)
        total, grad = 0.0, np.zeros_like(theta)

        def one(ci, bc, p):  # one solve: the bands, then the gradient from its eigenvectors
            b = bc.bands(p, keep_vectors=True)
            mse, dl_de = self._mse_terms(ci, b)
            _, gp = bc.backward(p, dl_de / nbs)
            return mse, gp

        for ci, (bc, (mse, gp)) in enumerate(zip(self.crystals, self._each_crystal(one, theta))):
            total += mse / nbs
            for t, s in enumerate(bc.types_of):
                e = self.fit.elements.index(s)
                first = next(i for i, c in enumerate(self.fit.crystals) if s in c.symbols)
                f = gp[t].copy()
                if first != ci:
                    f[0] *= self.fit.norm_vol[ci] / self.fit.norm_vol[first]
                grad[e] += f
        return total, grad

    def close(self):
        for bc in self.crystals:
            bc.close()


def write_band_structure(path, kpts, bands):
    """bandStruct_<i>.dat: |k| then the bands, "% .5f " each (write.c:54-66)."""
    with open(path, "w") as f:
        for k, row in zip(np.asarray(kpts), np.asarray(bands)):
            f.write("% .5f " % float(np.sqrt(k @ k)))
            f.write("".join("% .5f " % float(e) for e in row))
            f.write("\n")


_SEPARATION = "\n\n" + "*" * 63 + "\n\n"        # write.c:175-179


def write_kpoints(path, kpts):
    """kpoints_<i>.dat: x y z |k| per k-point, "% .10f" each (write.c:155-160)."""
    with open(path, "w") as f:
        for k in np.asarray(kpts):
            f.write("% .10f % .10f % .10f % .10f\n" % (k[0], k[1], k[2], float(np.sqrt(k @ k))))


def _pseudo_params(fit, theta):
    """write.c:109-125: per crystal, per atom, the symbol and 4 parameters."""
    out = []
    for ci, c in enumerate(fit.crystals):
        if ci:
            out.append("\n")
        out.append("\nBand structure %d\n" % ci)
        for s in c.symbols:
            p = fit_atom_params(fit, theta, ci, s)
            out.append("\n%s" % s + "".join(" % .8f" % v for v in p))
    return "".join(out)


def _iteration(fit, theta, mse, it, n_iterations):
    """write.c:72-80."""
    text = (_SEPARATION if it != 0 else "") + "Iteration %d\nMSE % .5f\n" % (it, mse)
    text += _pseudo_params(fit, theta)
    if it == n_iterations:
        text += _SEPARATION
    return text


def _input_summary(fit, n_iterations, nbv):
    """write.c:128-152."""
    out = ["INPUT\n\n",
           "The number of band structures fit to was: %d\n" % len(fit.crystals),
           "The kinetic energy scaling was: % .4f\n" % fit.ke_scale,
           "The total number of iterations was: %d\n" % n_iterations,
           "The beta used was: % .1f\n\n" % fit.beta,
           "The atoms were place at the following positions:\n\n"]
    for c in fit.crystals:
        for s, t in zip(c.symbols, c.tau):
            out.append("%s %.5f %.5f %.5f\n" % (s, t[0], t[1], t[2]))
    for ci, c in enumerate(fit.crystals):
        out += ["\nBand structure %d\n" % ci,
                "The number of atoms in the cell was: %d\n" % len(c.symbols),
                "The number of bands calculated was: %d\n" % c.ne,
                "The number of k-points that were used to fit the pseudopotentials to was: "
                "%d\n" % len(c.kpts),
                "The maximum kinetic energy was: % .3f\n" % c.max_ke,
                "The number of basis functions used was: %d\n" % nbv[ci]]
    out.append(_SEPARATION)
    return "".join(out)


def write_results(directory, fit, theta, bands, best_mse, n_iterations, nbv):
    """The files of writeResults and calcRealSpacePotential (write.c:7-69,
    pot.c:21-83): kpoints_<i>.dat, output.dat, best_<Sym>_<i>_Params.dat,
    bandStruct_<i>.dat and pot_<Sym>_<i>.dat."""
    import time

    from .binding import form_factor_table

    d = str(directory)
    for ci, c in enumerate(fit.crystals):
        write_kpoints(os.path.join(d, "kpoints_%d.dat" % ci), c.kpts)
    with open(os.path.join(d, "output.dat"), "w") as f:
        f.write(time.ctime() + "\n" + _SEPARATION)
        f.write("The best mean squared error found was: % .5f\n" % best_mse)
        f.write(_pseudo_params(fit, theta) + _SEPARATION)
        f.write(_input_summary(fit, n_iterations, nbv))
    for ci, c in enumerate(fit.crystals):
        for s in c.symbols:
            p = fit_atom_params(fit, theta, ci, s)
            with open(os.path.join(d, "best_%s_%d_Params.dat" % (s, ci)), "w") as f:
                f.write("".join("% .8f\n" % v for v in p))
        write_band_structure(os.path.join(d, "bandStruct_%d.dat" % ci), c.kpts, bands[ci])
        for s in c.symbols:
            r, v = form_factor_table(fit_atom_params(fit, theta, ci, s), c.vol_per_atom)
            with open(os.path.join(d, "pot_%s_%d.dat" % (s, ci)), "w") as f:
                f.write("".join("%g %g\n" % (x, y) for x, y in zip(r, v)))


def run_fit(directory, steps=None, lr=1e-3, fitter=None, log_every=10):
    """Fit the form-factor parameters of the run in ``directory`` with Adam on
    the GPU gradient, in place of the reference's Monte Carlo search
    (fit.c:9-69): reads its inputs, writes iterations.dat every log_every
    steps as it does, and at the end its result files (``write_results``)
    for the best parameters found.  The step of each parameter is lr times
    its initial magnitude (at least 0.01).  steps defaults to input.par's
    nIterations.  Returns (best parameters, best objective)."""
    import time

    d = str(directory)
    fit = read_fit_inputs(d)
    steps = fit.n_iterations if steps is None else int(steps)
    bf = fitter(fit) if fitter is not None else BulkFit(fit)
    theta = np.array(fit.params, dtype=np.float64)
    scale = lr * np.maximum(np.abs(theta), 0.01)
    m, v = np.zeros_like(theta), np.zeros_like(theta)
    b1, b2, eps = 0.9, 0.999, 1e-12
    val, grad = bf.objective_and_grad(theta)
    best, best_theta = val, theta.copy()
    with open(os.path.join(d, "iterations.dat"), "w") as f:
        f.write(time.ctime() + "\n" + _SEPARATION + _iteration(fit, theta, val, 0, steps))
    for it in range(1, steps + 1):
        m = b1 * m + (1 - b1) * grad
        v = b2 * v + (1 - b2) * grad * grad
        mh, vh = m / (1 - b1 ** it), v / (1 - b2 ** it)
        theta = theta - scale * mh / (np.sqrt(vh) + eps)
        val, grad = bf.objective_and_grad(theta)
        if val < best:
            best, best_theta = val, theta.copy()
        if it % log_every == 0:
            with open(os.path.join(d, "iterations.dat"), "a") as f:
                f.write(_iteration(fit, theta, val, it, steps))
    with open(os.path.join(d, "iterations.dat"), "a") as f:
        f.write(time.ctime() + "\n")
    bands = bf.band_structures(best_theta)
    nbv = [bc.nbv for bc in bf.crystals]
    write_results(d, fit, best_theta, bands, best, steps, nbv)
    if fitter is None:
        bf.close()
    return best_theta, best


def _autograd():
    import torch

    class BandStructureMSE(torch.autograd.Function):
        """The fit objective of ``BulkFit`` as a torch function of the fit
        parameters (len(elements) x 4, float64)."""

        @staticmethod
        def forward(ctx, theta, fit):
            val, grad = fit.objective_and_grad(theta.detach().cpu().numpy())
            ctx.save_for_backward(torch.as_tensor(grad, dtype=theta.dtype))
            return theta.new_tensor(val)

        @staticmethod
        def backward(ctx, g):
            (grad,) = ctx.saved_tensors
            return g * grad.to(g.device), None

    return BandStructureMSE


def __getattr__(name):
    if name == "BandStructureMSE":
        return _autograd()
    raise AttributeError(name)


def main(argv=None):
    """python -m semi_empirical_pseudopotentials_gb300.bulk RUN_DIR [--steps N] [--lr X]"""
    import argparse

    p = argparse.ArgumentParser(description="Fit form-factor parameters to bulk band "
                                "structures on the GPU (the inputs and outputs of "
                                "pseudopotFitting/).")
    p.add_argument("directory")
    p.add_argument("--steps", type=int, default=None,
                   help="optimiser steps (default: input.par's nIterations)")
    p.add_argument("--lr", type=float, default=1e-3,
                   help="step per parameter, relative to its initial magnitude")
    a = p.parse_args(argv)
    theta, best = run_fit(a.directory, a.steps, a.lr)
    print("The best mean squared error found was: % .5f" % best)
    return 0


__all__ = ["Crystal", "FitInputs", "read_fit_inputs", "fit_atom_params", "basis", "BulkCrystal",
           "BulkFit", "band_weights", "write_band_structure", "write_kpoints", "write_results",
           "run_fit", "BandStructureMSE", "SepError"]

if __name__ == "__main__":
    raise SystemExit(main())
