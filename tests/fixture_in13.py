"""Inputs of the reference's In13_P16 fixture (filterStrainCube/test/In13_P16)
rebuilt from tests/golden/in13_p16.npz the way the reference builds them:
centre the atoms (filter/read.c:16-30), box rint(0.5 extent + 5)
(filter/init.c:90-114), shift each table by its last value
(filter/read.c:105-108), V(r) with the per-atom strain scale
(filterStrainCube/interpolate.c:11-25), k^2 (filter/init.c:124-144)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load():
    g = np.load(os.path.join(GOLDEN, "in13_p16.npz"))
    d = {k: g[k] for k in g.files}
    xyz = np.array(d["xyz_raw"], dtype=np.float64)
    for k in range(3):  # mean summed in atom order, as the reference does
        m = 0.0
        for v in xyz[:, k]:
            m += v
        xyz[:, k] -= m / len(xyz)
    half = [float(np.rint(0.5 * (xyz[:, k].max() - xyz[:, k].min()) + 5.0)) for k in range(3)]
    dims = tuple(int(v) for v in d["dims"])
    steps = tuple(2.0 * h / n for h, n in zip(half, dims))
    tab_v = np.array(d["tab_v"])
    for t in range(tab_v.shape[0]):
        n = int(d["tab_n"][t])
        if n > 0:
            tab_v[t, :n] -= tab_v[t, n - 1]
    ms = int(d["ms"])
    el = float(d["elmin"]) + np.arange(ms) * ((float(d["elmax"]) - float(d["elmin"])) / (ms - 1))
    d.update(xyz=xyz, half=half, dims=dims, steps=steps, mins=tuple(-h for h in half),
             dv=steps[0] * steps[1] * steps[2], tab_v_shifted=tab_v, el=el,
             seed=-1131359211)  # the seed of run.dat:53
    return d
