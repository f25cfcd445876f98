"""Golden fixture for the bulk band-structure path (pseudopotFitting/).

Run in a container that has the reference checkout (not on a GPU machine):

    python tests/golden/make_bulk_fixture.py [REFERENCE_CHECKOUT]

It copies the text of the reference's published fitting runs
(pseudopotFitting/TESTS/{zb_cdse,w_cdse,cdse}: the inputs, output.dat, the
band structures and k-point files the program wrote, and zb_cdse's
real-space tables) into tests/golden/bulk_fit.json.  Then, with
oracle/_ref/libfitref.so (the reference's pseudopotFitting sources compiled
by oracle/Makefile.ref), it computes each run's band structures at the
parameters printed in its output.dat, the reference's weighted and
unweighted objectives on them (fit.c:71-177) and its plane-wave bases, in
full precision, into tests/golden/bulk_ref.npz.
zb_cdse ran 0 Monte Carlo steps, so its band structure belongs to its input
parameters; w_cdse and cdse belong to the best parameters printed in
output.dat.
"""
import ctypes
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = ["zb_cdse", "w_cdse", "cdse"]
SKIP = ("pot_", "iterations", "run.dat", "w_", "zb_")
KEEP = ("pot_Cd_0.dat", "pot_Se_0.dat")      # zb_cdse only: the real-space tables


def main():
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
    from oracle.build_oracle import reference_dir

    ref = reference_dir(sys.argv[1] if len(sys.argv) > 1 else None)
    out = {}
    for run in RUNS:
        d = os.path.join(ref, "pseudopotFitting", "TESTS", run)
        files = {}
        for fn in sorted(os.listdir(d)):
            if fn.startswith(SKIP) and not (run == "zb_cdse" and fn in KEEP):
                continue
            with open(os.path.join(d, fn)) as f:
                files[fn] = f.read()
        out[run] = files
        print(run, sorted(files))
    with open(os.path.join(HERE, "bulk_fit.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    reference_objective()


# ---- full-precision band structures and objectives from the reference's own
# code (oracle/_ref/libfitref.so, built by oracle/Makefile.ref): the structs
# of pseudopotFitting/fit.h:37-70, filled from the run's inputs; the basis by
# its getRecipSpaceBasisVectors, calcBasisVectors and finalizeBasisStates
class Vec(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double),
                ("mag", ctypes.c_double)]


class Atom(ctypes.Structure):
    _fields_ = [("symbol", ctypes.c_char * 10), ("type", ctypes.c_int), ("pos", Vec),
                ("ppParams", ctypes.c_double * 4), ("fF", ctypes.c_double)]


class Param(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in ("nBandStructures", "nIterations", "nAtoms",
                                              "nAtomTypes", "nElectrons", "nKPoints", "nKPE")] +
                [(n, ctypes.c_int * 20) for n in ("nkp", "ne", "na", "nqp", "nbv", "nmbv")] +
                [(n, ctypes.c_double * 20) for n in ("s", "mke", "vol", "volPerAtom",
                                                     "normalizedVolPerAtom")] +
                [(n, ctypes.c_int) for n in ("nQpoints", "nBasisVectors", "nMaxBV")] +
                [(n, ctypes.c_double) for n in ("scale", "maxKE", "beta", "stepSize",
                                                "kineticEnergyScaling")])


def vec(v):
    x, y, z = (float(t) for t in v)
    return Vec(x, y, z, math.sqrt(x * x + y * y + z * z))


def reference_objective():
    import tempfile

    import numpy as np

    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from semi_empirical_pseudopotentials_gb300 import bulk
    from tests import fixture_bulk as fb

    lib = ctypes.CDLL(os.path.join(HERE, "..", "..", "oracle", "_ref", "libfitref.so"))
    lib.calcAllIndividualWeightedMSE.restype = ctypes.c_double
    lib.calcAllIndividualMSE.restype = ctypes.c_double
    res = {}
    for run in RUNS:
        with tempfile.TemporaryDirectory() as tmp:
            fit = bulk.read_fit_inputs(fb.materialise(run, tmp))
        best = fb.best_atom_params(run)
        nbs = len(fit.crystals)
        par = Param()
        par.nBandStructures = nbs
        par.kineticEnergyScaling = fit.ke_scale
        par.nElectrons = max(c.ne for c in fit.crystals)
        basis, kpts, atoms, exp = [], [], [], []
        for i, c in enumerate(fit.crystals):
            cell = (Vec * 3)(*[vec(r) for r in c.cell])
            g = (Vec * 3)()
            nmbv = lib.getRecipSpaceBasisVectors(cell, g, ctypes.c_double(c.max_ke))
            tmpbv = (Vec * nmbv)()
            nbv = lib.calcBasisVectors(tmpbv, g, ctypes.c_double(c.max_ke))
            bs = (Vec * nbv)()
            lib.finalizeBasisStates(bs, tmpbv, nmbv, ctypes.c_double(c.max_ke))
            basis += list(bs)
            kpts += [vec(k) for k in c.kpts]
            for a, sym in enumerate(c.symbols):
                at = Atom(symbol=sym.encode(), pos=vec(c.tau[a]))
                for j in range(4):
                    at.ppParams[j] = best[i][a][j]
                atoms.append(at)
            exp.append(np.asarray(c.exp_bands).ravel())
            par.na[i], par.ne[i], par.nkp[i], par.nbv[i] = len(c.symbols), c.ne, len(c.kpts), nbv
            res[f"{run}_nbv_{i}"] = nbv
            res[f"{run}_basis_{i}"] = np.array([[v.x, v.y, v.z] for v in bs])
        nkpe = sum(c.ne * len(c.kpts) for c in fit.crystals)
        n2 = sum(par.nbv[i] ** 2 for i in range(nbs))
        band = np.zeros(nkpe)
        ham = np.zeros(2 * n2)
        pot = np.zeros(2 * n2)
        energies = np.zeros(max(par.nbv[i] for i in range(nbs)))
        dp = ctypes.POINTER(ctypes.c_double)
        lib.calcBandStructure(band.ctypes.data_as(dp), ham.ctypes.data_as(dp),
                              pot.ctypes.data_as(dp), (Vec * len(basis))(*basis),
                              (Vec * len(kpts))(*kpts), energies.ctypes.data_as(dp),
                              (Atom * len(atoms))(*atoms), par)
        expb = np.concatenate(exp)
        res[f"{run}_bands"] = band
        res[f"{run}_weighted_mse"] = lib.calcAllIndividualWeightedMSE(
            band.ctypes.data_as(dp), expb.ctypes.data_as(dp), par)
        res[f"{run}_mse"] = lib.calcAllIndividualMSE(band.ctypes.data_as(dp),
                                                     expb.ctypes.data_as(dp), par)
        print(run, "weighted", res[f"{run}_weighted_mse"], "plain", res[f"{run}_mse"])
    np.savez_compressed(os.path.join(HERE, "bulk_ref.npz"), **res)


if __name__ == "__main__":
    main()
