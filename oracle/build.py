"""Builds the CPU oracle library (test infrastructure only).

The oracle is a C++ restatement of the reference algorithms used by tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker. It is compiled with plain g++ (no CUDA) and with floating-point
contraction disabled so that its FP32 decision arithmetic has exactly one
rounding per written operation.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtotri_oracle.so")
SOURCES = ["mesh.cpp", "volume.cpp", "backprojection.cpp", "rbf.cpp"]
HEADERS = ["oracle_common.h"]

CXXFLAGS = [
    "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
    "-ffp-contract=off", "-fno-fast-math", "-fno-finite-math-only",
    "-Wall", "-Wno-unknown-pragmas",
]


def _sources():
    return [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = _sources() + [os.path.join(HERE, h) for h in HEADERS] + [__file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the oracle if needed and returns the shared-library path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", *CXXFLAGS, *_sources(), "-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
