"""The filter's output files and the merge of several filter runs.

Writers (byte for byte the reference program's files, written by
libsep_gb300.so):
* ``write_outputs``: psi.dat (raw FP64 state blocks) and eval.dat
  ("%ld %.16g %g": index, E, sigma), filter/main.c:129-142;
* ``write_filter_outputs``: eval-filt-<tid>-<jns>.dat ("%ld %.16g %.16g":
  index, E, target) and psi-filt-<tid>-<jns>.dat, filter/filter.c:37-47.

Merge (combine_filter_outputs.py, the step between the filter and bse/):
``combine`` and the command line

    python -m semi_empirical_pseudopotentials_gb300.outputs RUN [RUN ...]
        (--ngrid N | --grid-source input.par) [--output-dir merged_filter]
        [--eval-name eval.dat] [--psi-name psi.dat] [--copy-conf]

take the script's arguments, run its checks with its messages and exit
codes, and write the same eval.par, psi.par, merge_manifest.txt and
conf.par.  The work is done by sep_combine_outputs in the native library;
the state blocks are copied by a team of threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .binding import SepError, lib

_ERR_ARG = -1
_ERR_IO = -7


class MergeError(RuntimeError):
    """Filter outputs that cannot be merged (combine_filter_outputs.py:30-31)."""


def _raise(status, merge=False):
    if status == 0:
        return
    msg = lib().sep_last_error().decode(errors="replace")
    if merge and status == _ERR_ARG:
        raise MergeError(msg)
    if status == _ERR_IO:
        raise OSError(msg)
    raise SepError(status, msg)


def _path(p):
    return os.fsencode(os.fspath(p))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def write_states(path, psi):
    """Raw FP64 state blocks, no header (psi.dat, psi-filt-*.dat)."""
    psi = _f64(psi)
    m = psi.shape[0] if psi.ndim > 1 else (1 if psi.size else 0)
    n = psi.size // m if m else 0
    _raise(lib().sep_write_states(_path(path), _dp(psi), m, n))


def write_eval(path, eval, sige):
    """eval.dat: "%ld %.16g %g" per state (filter/main.c:138-142)."""
    e, s = _f64(eval).ravel(), _f64(sige).ravel()
    if e.size != s.size:
        raise ValueError("eval and sige differ in length")
    _raise(lib().sep_write_eval(_path(path), _dp(e), _dp(s), e.size))


def write_filter_eval(path, eval, el):
    """eval-filt-*.dat: "%ld %.16g %.16g" per target (filter/filter.c:37-41)."""
    e, t = _f64(eval).ravel(), _f64(el).ravel()
    if e.size != t.size:
        raise ValueError("eval and el differ in length")
    _raise(lib().sep_write_filter_eval(_path(path), _dp(e), _dp(t), e.size))


def write_outputs(directory, psi, eval, sige):
    """psi.dat and eval.dat of a finished run (filter/main.c:129-142)."""
    d = Path(directory)
    write_states(d / "psi.dat", psi)
    write_eval(d / "eval.dat", eval, sige)


def write_filter_outputs(directory, tid, jns, psi, eval, el):
    """eval-filt-<tid>-<jns>.dat and psi-filt-<tid>-<jns>.dat of one start
    state's filter (filter/filter.c:37-47)."""
    d = Path(directory)
    write_filter_eval(d / f"eval-filt-{int(tid)}-{int(jns)}.dat", eval, el)
    write_states(d / f"psi-filt-{int(tid)}-{int(jns)}.dat", psi)


def read_ngrid_from_input(path) -> int:
    """nx*ny*nz from the first three integers of an input.par
    (combine_filter_outputs.py:125-145)."""
    n = C.c_long()
    _raise(lib().sep_read_grid_source(_path(path), C.byref(n)), merge=True)
    return int(n.value)


@dataclass(frozen=True)
class MergeResult:
    roots: list
    nstates: list
    total: int
    output_dir: Path


def combine(datasets, output_dir="merged_filter", *, ngrid, eval_name="eval.dat",
            psi_name="psi.dat", copy_conf=False) -> MergeResult:
    """Merge the runs in ``datasets`` (directories) into output_dir; raises
    MergeError with the script's message when they cannot be merged."""
    dirs = [_path(d) for d in datasets]
    if not dirs:
        raise MergeError("no datasets")
    arr = (C.c_char_p * len(dirs))(*dirs)
    counts = (C.c_long * len(dirs))()
    total = C.c_long()
    _raise(lib().sep_combine_outputs(len(dirs), arr, _path(eval_name), _path(psi_name),
                                     int(ngrid), _path(output_dir), int(bool(copy_conf)),
                                     counts, C.byref(total)), merge=True)
    return MergeResult([Path(d).resolve() for d in datasets], list(counts), int(total.value),
                       Path(output_dir).resolve())


def parse_args(argv=None):
    p = argparse.ArgumentParser(
        description="Combine several filter runs (eval.dat + psi.dat) into one "
                    "eval.par/psi.par pair for bse/.")
    p.add_argument("datasets", nargs="+",
                   help="Directories holding eval.dat and psi.dat of filter runs.")
    p.add_argument("--output-dir", default="merged_filter",
                   help="Directory for eval.par, psi.par and merge_manifest.txt.")
    p.add_argument("--grid-source",
                   help="An input.par whose first three integers are nx ny nz.")
    p.add_argument("--ngrid", type=int, help="Grid points per state (instead of --grid-source).")
    p.add_argument("--eval-name", default="eval.dat",
                   help="Eigenvalue file name inside each dataset directory.")
    p.add_argument("--psi-name", default="psi.dat",
                   help="State file name inside each dataset directory.")
    p.add_argument("--copy-conf", action="store_true",
                   help="Copy the first dataset's conf.par (all copies must match).")
    args = p.parse_args(argv)
    if (args.grid_source is None) == (args.ngrid is None):
        p.error("provide exactly one of --grid-source or --ngrid")
    if args.ngrid is not None and args.ngrid <= 0:
        p.error("--ngrid must be positive")
    return args


def main(argv=None) -> int:
    args = parse_args(argv)
    ngrid = args.ngrid if args.ngrid is not None else read_ngrid_from_input(args.grid_source)
    try:
        r = combine(args.datasets, args.output_dir, ngrid=ngrid, eval_name=args.eval_name,
                    psi_name=args.psi_name, copy_conf=args.copy_conf)
    except MergeError as exc:
        print(f"error: {exc}", file=sys.stderr)
        return 1
    sources = ", ".join(f"{root} ({n} states)" for root, n in zip(r.roots, r.nstates))
    print(f"Merged {len(r.roots)} datasets: {sources}")
    print(f"Total merged states: {r.total}")
    print(f"ngrid per state: {ngrid}")
    for name in ("eval.par", "psi.par", "merge_manifest.txt") + (
            ("conf.par",) if args.copy_conf else ()):
        print(f"Wrote {r.output_dir / name}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
