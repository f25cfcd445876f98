"""Golden fixture for the bulk band-structure path (pseudopotFitting/).

Run in a container that has the reference checkout (not on a GPU machine):

    python tests/golden/make_bulk_fixture.py /root/reference

It copies the text of the reference's published fitting runs
(pseudopotFitting/TESTS/{zb_cdse,w_cdse,cdse}: the inputs, output.dat, the
band structures and k-point files the program wrote, and zb_cdse's
real-space tables) into tests/golden/bulk_fit.json.
zb_cdse ran 0 Monte Carlo steps, so its band structure belongs to its input
parameters; w_cdse and cdse belong to the best parameters printed in
output.dat.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = ["zb_cdse", "w_cdse", "cdse"]
SKIP = ("pot_", "iterations", "run.dat", "w_", "zb_")
KEEP = ("pot_Cd_0.dat", "pot_Se_0.dat")      # zb_cdse only: the real-space tables


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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


if __name__ == "__main__":
    main()
