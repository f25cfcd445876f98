"""The filter's output files and the merge step, against the reference's own
files and its combine_filter_outputs.py run on the same inputs
(tests/golden/output_formats.json, made by make_output_fixtures.py).
Host-side code: no GPU needed."""
import base64
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from semi_empirical_pseudopotentials_gb300 import outputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fx():
    with open(os.path.join(ROOT, "tests", "golden", "output_formats.json")) as f:
        return json.load(f)


def columns(text):
    rows = [line.split() for line in text.splitlines() if line.strip()]
    return [np.array([float(r[k]) for r in rows]) for k in (1, 2)]


def test_eval_dat_bytes_match_reference_file(fx, tmp_path):
    # In13_P16/eval.dat as the reference program wrote it ("%ld %.16g %g")
    e, s = columns(fx["in13_eval_dat"])
    assert e.size == 158
    outputs.write_eval(tmp_path / "eval.dat", e, s)
    assert (tmp_path / "eval.dat").read_bytes() == fx["in13_eval_dat"].encode()


def test_eval_filt_bytes_match_reference_file(fx, tmp_path):
    e, t = columns(fx["in13_eval_filt_0_0"])
    outputs.write_filter_outputs(tmp_path, 0, 0, np.zeros((e.size, 4)), e, t)
    assert (tmp_path / "eval-filt-0-0.dat").read_bytes() == fx["in13_eval_filt_0_0"].encode()
    assert (tmp_path / "psi-filt-0-0.dat").read_bytes() == bytes(8 * 4 * e.size)


@pytest.mark.parametrize("m,n", [(0, 60), (3, 60), (9, 1 << 20)])
def test_state_file_is_raw_doubles(tmp_path, m, n):
    # 9 x 2^20 doubles = 72 MiB: more than one 64 MiB piece
    psi = np.random.default_rng(m).standard_normal((m, n))
    outputs.write_outputs(tmp_path, psi, np.arange(m) * -0.1, np.full(m, 1e-7))
    got = np.fromfile(tmp_path / "psi.dat", dtype=np.float64)
    assert got.size == m * n and np.array_equal(got, psi.ravel())
    lines = (tmp_path / "eval.dat").read_text().splitlines()
    assert lines == [f"{k} {-0.1 * k:.16g} 1e-07" for k in range(m)]


def test_writer_reports_unwritable_path(tmp_path):
    with pytest.raises(OSError, match="No such file or directory"):
        outputs.write_eval(tmp_path / "no" / "eval.dat", [1.0], [0.0])


def materialise(fx, root):
    for name, files in fx["datasets"].items():
        if "->" in files:                       # a symbolic link to another dataset
            os.symlink(base64.b64decode(files["->"]).decode(), root / name)
            continue
        os.makedirs(root / name, exist_ok=True)
        for fn, data in files.items():
            (root / name / fn).write_bytes(base64.b64decode(data))


def last_line(text):
    return text.strip().splitlines()[-1]


CASES = ["merge3", "grid_source", "names", "names_missing", "conf_differs", "psi_size",
         "not_sequential", "two_columns", "non_numeric", "hex_float", "empty_eval", "missing_psi",
         "missing_dir", "ngrid_mismatch", "copy_conf_missing", "grid_nonpositive",
         "symlink_and_dotdot", "absolute_names", "no_grid", "ngrid_zero"]


@pytest.mark.parametrize("name", CASES)
def test_merge_matches_reference_script(fx, tmp_path, monkeypatch, capsys, name):
    case = fx["cases"][name]
    root = tmp_path.resolve()
    materialise(fx, root)
    monkeypatch.chdir(root)
    args = [a.replace("{ROOT}", str(root)) for a in case["args"]]
    rc, raised = None, None
    try:
        rc = outputs.main(args)
    except SystemExit as e:          # argparse errors: exit 2
        rc = e.code
    except outputs.MergeError as e:  # the script lets this one escape (exit 1)
        rc, raised = 1, str(e)
    out, err = capsys.readouterr()
    out, err = out.replace(str(root), "{ROOT}"), err.replace(str(root), "{ROOT}")
    assert rc == case["rc"]
    if rc == 2:
        assert last_line(err).split("error: ", 1)[1] == \
            last_line(case["stderr"]).split("error: ", 1)[1]
    elif raised is not None:
        assert last_line(case["stderr"]).endswith("MergeError: " + raised)
    else:
        assert out == case["stdout"]
        assert err == case["stderr"]
    outdir = root / (args[args.index("--output-dir") + 1] if "--output-dir" in args
                     else "merged_filter")
    got = {}
    if outdir.is_dir():
        for fn in sorted(os.listdir(outdir)):
            data = (outdir / fn).read_bytes()
            if fn == "merge_manifest.txt":
                data = data.replace(str(root).encode(), b"{ROOT}")
            got[fn] = data
    want = {fn: base64.b64decode(v) for fn, v in case["files"].items()}
    assert sorted(got) == sorted(want)
    for fn in want:
        assert got[fn] == want[fn], fn


def test_merge_command_line(fx, tmp_path):
    case = fx["cases"]["merge3"]
    root = tmp_path.resolve()
    materialise(fx, root)
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "semi_empirical_pseudopotentials_gb300.outputs"] +
                       case["args"], cwd=root, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert r.stdout.replace(str(root), "{ROOT}") == case["stdout"]
    assert (root / "merged_filter" / "psi.par").read_bytes() == \
        base64.b64decode(case["files"]["psi.par"])


def test_merge_of_large_blocks_keeps_order(tmp_path):
    # blocks larger than the 8 MiB copy chunk, many states over the thread team
    n = (1 << 20) + 5
    rng = np.random.default_rng(5)
    blocks = {}
    for d, m in (("a", 7), ("b", 6)):
        (tmp_path / d).mkdir()
        e = rng.permutation(m) * 0.01 - (0.005 if d == "b" else 0.0)
        psi = rng.standard_normal((m, n))
        outputs.write_outputs(tmp_path / d, psi, e, np.full(m, 1e-6))
        for k in range(m):
            blocks[(d, k)] = (e[k], psi[k])
    r = outputs.combine([tmp_path / "a", tmp_path / "b"], tmp_path / "out", ngrid=n)
    assert r.total == 13 and r.nstates == [7, 6]
    order = sorted(blocks, key=lambda k: (blocks[k][0], 1e-6, k[0], k[1]))
    got = np.fromfile(tmp_path / "out" / "psi.par", dtype=np.float64).reshape(13, n)
    for j, key in enumerate(order):
        assert np.array_equal(got[j], blocks[key][1])
