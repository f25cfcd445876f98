"""Build recipe for the oracle (test infrastructure only).

* ``liboracle.so``  -- the C restatement (sep_oracle.c + fft_cpu.c); built on
  every machine, because the tests and the CPU baseline need it.
* ``_ref/``         -- the reference's own filter sources compiled in place by
  Makefile.ref; built only where the reference checkout exists.

The product library never links or loads anything built here.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir(ref=None):
    """The reference checkout: `ref` when given, else $SEP_REFERENCE, else a
    directory named ``reference`` beside this repository's root."""
    if ref:
        return ref
    env = os.environ.get("SEP_REFERENCE")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def openblas_path():
    """Path of the ILP64 OpenBLAS that numpy bundles (scipy_-prefixed LAPACK)."""
    import numpy

    base = os.path.dirname(os.path.dirname(numpy.__file__))
    for pat in ("numpy.libs/libscipy_openblas64_*.so*", "numpy/.libs/libscipy_openblas64_*.so*"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


def build_oracle(verbose=False):
    src = [os.path.join(HERE, "sep_oracle.c"), os.path.join(HERE, "fft_cpu.c")]
    out = os.path.join(HERE, "liboracle.so")
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in
                                   src + [os.path.join(HERE, "sep_oracle.h"),
                                          os.path.join(HERE, "fft_cpu.h")]):
        return out
    cmd = ["gcc", "-std=gnu11", "-O3", "-fopenmp", "-fPIC", "-ffp-contract=off", "-shared",
           "-o", out] + src + ["-lm", "-ldl"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_ref(ref=None, verbose=False):
    """Compile the reference's sources into _ref/ when the checkout exists."""
    ref = reference_dir(ref)
    if not os.path.isdir(os.path.join(ref, "filter")):
        return None
    blas = openblas_path()
    if blas is None:
        return None
    cmd = ["make", "-s", "-f", "Makefile.ref", "-j8", "REF=" + ref, "OPENBLAS=" + blas]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd, cwd=HERE, stdout=None if verbose else subprocess.DEVNULL)
    return os.path.join(HERE, "_ref")


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True) or "reference checkout not present: _ref not built",
          file=sys.stderr)
