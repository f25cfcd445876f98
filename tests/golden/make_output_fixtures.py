"""Golden fixtures for the filter's output files and the merge step.

Run in a container that has the reference checkout (not on a GPU machine):

    python tests/golden/make_output_fixtures.py [REFERENCE_CHECKOUT]

It writes tests/golden/output_formats.json with
* the text of In13_P16's eval.dat (filterStrainCube/main.c:163-166,
  "%ld %.16g %g") and of one eval-filt file (filterStrainCube/filter.c,
  "%ld %.16g %.16g"), as written by the reference program;
* a set of small filter-output directories (eval.dat, psi.dat, input.par,
  conf.par; seeded values with ties in energy and sigma, CRLF lines, blank
  lines, extra columns, exotic number forms), and for each merge case the
  arguments, the exit code, stdout and stderr, and every file the
  reference's combine_filter_outputs.py wrote.  Paths under the temporary
  root are replaced by "{ROOT}".
"""
import base64
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

NGRID = 60          # 3 x 4 x 5
HERE = os.path.dirname(os.path.abspath(__file__))


def b64(data):
    return base64.b64encode(data).decode()


def eval_text(rows, fmt="{} {:.16g} {:g}\n"):
    return "".join(fmt.format(*r) for r in rows).encode()


def psi_bytes(rng, nstates):
    return rng.standard_normal((nstates, NGRID)).astype(np.float64).tobytes()


def datasets():
    rng = np.random.default_rng(20261203)
    inp = b"3\n4\n5\n10\n16\n1024\n-0.23\n-0.05\n6\nzincblende\nInP\n"
    conf = b"2\nIn 0.0 0.0 0.0\nP 2.0 2.0 2.0\n"
    d = {}
    d["A"] = {
        "eval.dat": eval_text([(0, -0.30, 1e-3), (1, -0.25, 2e-3), (2, -0.25, 1e-3),
                               (3, -0.10, 5e-4), (4, 0.05, 3e-3)]),
        "psi.dat": psi_bytes(rng, 5), "input.par": inp, "conf.par": conf}
    # ties with A in (energy, sigma), a signed zero against an unsigned one
    d["B"] = {
        "eval.dat": eval_text([(0, -0.25, 1e-3), (1, -0.0, 7e-4), (2, 0.0, 7e-4),
                               (3, -0.3461655492210728, 0.00158923)]),
        "psi.dat": psi_bytes(rng, 4), "input.par": inp, "conf.par": conf}
    # no input.par or conf.par; CRLF endings, a blank line, tabs, a fourth
    # column, a signed index and number forms that Python's int()/float() accept
    d["C"] = {
        "eval.dat": (b"0 1e-05 2.5e-07\r\n\r\n  1\t-0.2500000000000001 1E-3 extra\r\n"
                     b"+2 1_0.5e-2 0.000_1\r\n3 -inf 0\r\n"),
        "psi.dat": psi_bytes(rng, 4)}
    # other file names
    d["D"] = {"eval-x.dat": eval_text([(0, -0.2, 1e-4), (1, -0.15, 2e-4)]),
              "psi-x.dat": psi_bytes(rng, 2), "conf.par": conf}
    d["E_conf"] = dict(d["A"], **{"conf.par": conf + b"Cd 1.0 1.0 1.0\n"})
    d["F_psi_short"] = dict(d["A"], **{"psi.dat": psi_bytes(rng, 4)})
    d["G_order"] = {"eval.dat": eval_text([(0, -0.3, 1e-3), (2, -0.2, 1e-3), (1, -0.1, 1e-3)]),
                    "psi.dat": psi_bytes(rng, 3)}
    d["H_cols"] = {"eval.dat": b"0 -0.3 1e-3\n1 -0.2\n", "psi.dat": psi_bytes(rng, 2)}
    d["I_text"] = {"eval.dat": b"0 -0.3 1e-3\n1 abc 1e-3\n", "psi.dat": psi_bytes(rng, 2)}
    d["J_empty"] = {"eval.dat": b"\n  \n\t\n", "psi.dat": b""}
    d["K_nopsi"] = {"eval.dat": eval_text([(0, -0.3, 1e-3)])}
    d["L_hex"] = {"eval.dat": b"0 0x1p-3 1e-3\n", "psi.dat": psi_bytes(rng, 1)}
    d["M_grid"] = {"input.par": b"3 4 0\n"}
    d["N_link"] = {"->": b"B"}                       # a symbolic link to B
    return d


CASES = [
    ("merge3", ["A", "B", "C", "--ngrid", "60", "--copy-conf"]),
    ("grid_source", ["A", "B", "--grid-source", "A/input.par", "--output-dir", "out/deeper"]),
    ("names", ["D", "--ngrid", "60", "--eval-name", "eval-x.dat", "--psi-name", "psi-x.dat"]),
    ("names_missing", ["A", "D", "--ngrid", "60", "--eval-name", "eval-x.dat",
                       "--psi-name", "psi-x.dat"]),
    ("conf_differs", ["A", "E_conf", "--ngrid", "60"]),
    ("psi_size", ["F_psi_short", "--ngrid", "60"]),
    ("not_sequential", ["G_order", "--ngrid", "60"]),
    ("two_columns", ["H_cols", "--ngrid", "60"]),
    ("non_numeric", ["I_text", "--ngrid", "60"]),
    ("hex_float", ["L_hex", "--ngrid", "60"]),
    ("empty_eval", ["J_empty", "--ngrid", "60"]),
    ("missing_psi", ["K_nopsi", "--ngrid", "60"]),
    ("missing_dir", ["A", "no/such/dir", "--ngrid", "60"]),
    ("ngrid_mismatch", ["A", "--ngrid", "61"]),
    ("copy_conf_missing", ["C", "A", "--ngrid", "60", "--copy-conf"]),
    ("grid_nonpositive", ["A", "--grid-source", "M_grid/input.par"]),
    ("symlink_and_dotdot", ["N_link", "C/../A", "--ngrid", "60"]),
    ("absolute_names", ["D", "--ngrid", "60", "--eval-name", "{ROOT}/D/eval-x.dat",
                        "--psi-name", "{ROOT}/D/psi-x.dat", "--output-dir", "{ROOT}/abs_out"]),
    ("no_grid", ["A"]),
    ("ngrid_zero", ["A", "--ngrid", "0"]),
]


def materialise(root, sets):
    """Writes the datasets under root; {"->": target} makes a symbolic link."""
    for name, files in sets.items():
        if "->" in files:
            os.symlink(files["->"].decode(), os.path.join(root, name))
            continue
        os.makedirs(os.path.join(root, name), exist_ok=True)
        for fn, data in files.items():
            with open(os.path.join(root, name, fn), "wb") as f:
                f.write(data)


def run_case(script, sets, args):
    with tempfile.TemporaryDirectory() as tmp:
        root = str(Path(tmp).resolve())
        materialise(root, sets)
        args = [a.replace("{ROOT}", root) for a in args]
        r = subprocess.run([sys.executable, script] + args, cwd=root, capture_output=True,
                           text=True)
        outdir = None
        if "--output-dir" in args:
            outdir = os.path.join(root, args[args.index("--output-dir") + 1])
        else:
            outdir = os.path.join(root, "merged_filter")
        files = {}
        if os.path.isdir(outdir):
            for fn in sorted(os.listdir(outdir)):
                data = open(os.path.join(outdir, fn), "rb").read()
                if fn == "merge_manifest.txt":
                    data = data.replace(root.encode(), b"{ROOT}")
                files[fn] = b64(data)
        # the script's own location (in tracebacks) is replaced by {SCRIPT_DIR}
        sdir = os.path.dirname(os.path.abspath(script))
        return {"rc": r.returncode, "stdout": r.stdout.replace(root, "{ROOT}"),
                "stderr": r.stderr.replace(root, "{ROOT}").replace(sdir, "{SCRIPT_DIR}"),
                "files": files}


def main():
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
    from oracle.build_oracle import reference_dir

    ref = reference_dir(sys.argv[1] if len(sys.argv) > 1 else None)
    script = os.path.join(ref, "combine_filter_outputs.py")
    in13 = os.path.join(ref, "filterStrainCube", "test", "In13_P16")
    sets = datasets()
    out = {
        "ngrid": NGRID,
        "in13_eval_dat": open(os.path.join(in13, "eval.dat"), "rb").read().decode(),
        "in13_eval_filt_0_0": open(os.path.join(in13, "eval-filt-0-0.dat"), "rb").read().decode(),
        "datasets": {k: {fn: b64(v) for fn, v in files.items()} for k, files in sets.items()},
        "cases": {},
    }
    for name, args in CASES:
        out["cases"][name] = dict(args=args, **run_case(script, sets, args))
        print(name, out["cases"][name]["rc"], out["cases"][name]["stderr"].strip()[-100:])
    with open(os.path.join(HERE, "output_formats.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
