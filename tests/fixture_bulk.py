"""The reference's published bulk fitting runs (pseudopotFitting/TESTS
zb_cdse, w_cdse, cdse; tests/golden/bulk_fit.json), written back into a
directory, and the parameters each band structure was computed with."""
import json
import os
import re

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def runs():
    with open(os.path.join(GOLDEN, "bulk_fit.json")) as f:
        return json.load(f)


def materialise(run, directory):
    os.makedirs(directory, exist_ok=True)
    for fn, text in runs()[run].items():
        with open(os.path.join(directory, fn), "w") as f:
            f.write(text)
    return directory


def best_atom_params(run):
    """Per band structure, the per-atom parameters printed under "The best
    mean squared error found was" in output.dat (write.c:109-125)."""
    text = runs()[run]["output.dat"]
    part = text.split("The best mean squared error found was:")[1].split("INPUT")[0]
    out, cur = [], None
    for line in part.splitlines():
        if line.startswith("Band structure"):
            cur = []
            out.append(cur)
        elif cur is not None and re.match(r"^[A-Z][a-z]?\s", line):
            t = line.split()
            cur.append([float(x) for x in t[1:5]])
    return [np.array(c) for c in out]


def published_bands(run, i):
    rows = np.loadtxt(runs()[run][f"bandStucture_{i}.dat"].splitlines())
    return rows[:, 0], rows[:, 1:]
