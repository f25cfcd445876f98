"""Build libsep_gb300.so (CUDA kernels for sm_103a + host code + C ABI) in-tree.

nvcc compiles the .cu translation units for sm_103a only; g++ compiles the
host numerics with -ffp-contract=off (they must match the reference bit for
bit); gcc compiles the fd.h-compatible C layer.  Objects go to _build/, the
library next to this file.  Translation units compile in parallel and are
skipped when up to date.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsep_gb300.so")
COMPAT_LIB = os.path.join(HERE, "libsep_fdcompat.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]
CUDA_UNITS = ["sep_pass_f64.cu", "sep_pass_f32.cu", "sep_pass_f64_v1.cu", "sep_pass_f32_v1.cu",
              "sep_pass_dd.cu", "sep_pass_dd_g0.cu", "sep_pass_dd_g1.cu", "sep_pass_dd_g2.cu",
              "sep_pass_dd_g3.cu",
              "sep_xy_f32.cu", "sep_sp_f32.cu",
              "sep_kernels.cu", "sep_ctx.cu",
              "sep_api.cu", "sep_vbuild.cu", "sep_noalloc.cu",
              "sep_ozaki.cu", "sep_bulk.cu", "sep_spinor.cu", "sep_spinor_path.cu",
              "sep_eigh.cu", "sep_heevb.cu"]
CXX_UNITS = ["sep_host.cpp", "sep_adjoint.cpp", "sep_io.cpp", "sep_spinor_host.cpp"]


def cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    deps = _headers()
    tasks = []
    objs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            tasks.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    for u in CXX_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            tasks.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread",
                          "-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, verbose), tasks))
    if tasks or not os.path.exists(LIB):
        libdir = os.path.join(cuda, "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(cuda, "lib")
        # --no-undefined: a symbol missing from the objects fails the build
        # here, not the first dlopen on a GPU machine
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-L" + libdir, "-lcusolver", "-Xcompiler", "-pthread", "-Xlinker",
              "-rpath," + libdir, "-Xlinker", "--no-undefined"], verbose)
    compat_src = os.path.join(CSRC, "sep_fdcompat.c")
    if os.path.exists(compat_src) and _stale(COMPAT_LIB, compat_src, deps + [LIB]):
        _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
              compat_src, "-o", COMPAT_LIB, "-L" + HERE, "-lsep_gb300",
              "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
