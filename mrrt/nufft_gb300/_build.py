"""Build libgbnufft.so in-tree with nvcc for sm_103a.

The library is a plain C-ABI shared object (``include/gbnufft.h``); it links
the CUDA runtime and cuFFT and nothing from PyTorch.  Translation units are
compiled in parallel and linked once.

``build(checked=True)`` compiles the same sources with ``GBN_CHECKED`` into
``libgbnufft_checked.so``: every global index a kernel forms from plan data
is tested against its buffer's extent, a failed test is recorded in the
plan's status word (``gbn_debug_check_status``) and the access skipped.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "libgbnufft.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED_PATH = os.path.join(HERE, "libgbnufft_checked.so")

SOURCES = ["gbn_plan.cu", "gbn_gather.cu", "gbn_spread.cu", "gbn_padcrop.cu", "gbn_dtft.cu", "gbn_grad.cu",
           "gbn_noalloc.cu", "gbn_coef.cu", "gbn_bin.cu", "gbn_sort.cu", "gbn_colfft.cu", "gbn_rowfft.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def _cuda_lib_dir():
    root = os.path.dirname(os.path.dirname(nvcc()))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcufft.so")):
            return d
    return os.path.join(root, "lib64")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, checked=False):
    """Compile every translation unit (in parallel) and link libgbnufft.so
    (or, with ``checked``, libgbnufft_checked.so)."""
    build_dir = BUILD_CHECKED if checked else BUILD
    lib_path = LIB_CHECKED_PATH if checked else LIB_PATH
    defines = ["-DGBN_CHECKED"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(os.path.dirname(HERE)), "include", "gbnufft.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + ARCH + FLAGS + defines + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(lib_path, objs):
        tmp = lib_path + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + [
            "-L" + _cuda_lib_dir(), "-lcufft", "-lcudart"]
        run(cmd)
        os.replace(tmp, lib_path)
    return lib_path


def build_all(force=False, verbose=False):
    """Both libraries, the normal and the checked build, compiled together."""
    with ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build, force, verbose, False)
        b = ex.submit(build, force, verbose, True)
        return a.result(), b.result()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
