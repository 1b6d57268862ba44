"""Builds libtotri_gb300.so (all CUDA kernels + the C ABI) for sm_103a.

Each translation unit in csrc/ is compiled by nvcc in parallel into _build/,
then linked into totri_gb300/_build/libtotri_gb300.so with the CUDA runtime
linked statically. The build is incremental (object files newer than their
source and the shared headers are reused).

With TOTRI_BOUNDS_CHECK=1 in the environment the bounds-checking variant is
built instead, into _build_check/ (-DTOTRI_BOUNDS_CHECK: the indices the
kernels take from device data are checked, an out-of-range one raises a device
status bit and is clamped), and the loader picks that library.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_NAME = "libtotri_gb300.so"


def bounds_check():
    """True when TOTRI_BOUNDS_CHECK=1 selects the bounds-checking build."""
    return os.environ.get("TOTRI_BOUNDS_CHECK", "") not in ("", "0")


BUILD_DIR = os.path.join(PKG, "_build_check" if bounds_check() else "_build")
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
CHECK_FLAGS = ["-DTOTRI_BOUNDS_CHECK"] if bounds_check() else []

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
    "-I" + INCLUDE, "-I" + CSRC,
]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else "nvcc"


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    deps = [src, __file__] + _headers()
    if os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *CHECK_FLAGS, *extra, "-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    if verbose and res.stderr.strip():
        print(res.stderr, file=sys.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, ptxas_info=False, jobs=None):
    """Compiles every kernel source and links the C-ABI library; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose or ptxas_info), sources))
    if os.path.exists(LIB_PATH) and all(
            os.path.getmtime(o) <= os.path.getmtime(LIB_PATH) for o in objs):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", *objs, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
