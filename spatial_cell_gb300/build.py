"""Builds libspatialcell.so and its driver sc_run in-tree for sm_103a (GB300).

    python -m spatial_cell_gb300.build [--force]

Each translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``, ``-fmad=false`` so no
multiply-add is fused and every operation rounds as written), the host C++
with g++, and the objects are linked into spatial_cell_gb300/_lib/.  The
top-level CMakeLists.txt builds the same library and driver with the same
flags; this script calls the compilers directly so it runs where CMake is
not installed.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libspatialcell.so")
DRIVER = os.path.join(OUT_DIR, "sc_run")
DRIVER_SRC = os.path.join(HERE, "driver", "sc_run.cpp")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["sc_grid.cu", "sc_step.cu", "sc_sim.cu", "sc_noalloc.cu", "sc_observe.cu"]
CPP_SOURCES = ["sc_host.cpp"]
HEADERS = ["scmath.h", "sc_dev.cuh", "sc_launch.h", "sc_json.hpp", "sc_tile.cuh", "sc_gen.h"]


def _deps():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS] + [os.path.join(INCLUDE, "spatialcell.h")]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def up_to_date():
    if not (os.path.exists(LIB) and os.path.exists(DRIVER)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(DRIVER))
    return all(os.path.getmtime(d) <= t for d in _deps() + [DRIVER_SRC])


def build(force=False, verbose=False):
    """Compiles and links the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = ["-I", CSRC, "-I", INCLUDE]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(OUT_DIR, f.replace(".cu", ".o"))
        jobs.append((obj, [NVCC, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
                           "-Xptxas", "-v" if verbose else "-O3", *inc, "-c", os.path.join(CSRC, f), "-o", obj]))
    for f in CPP_SOURCES:
        obj = os.path.join(OUT_DIR, f.replace(".cpp", ".o"))
        jobs.append((obj, ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", *inc, "-c",
                           os.path.join(CSRC, f), "-o", obj]))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *[j[0] for j in jobs]])
    os.replace(tmp, LIB)
    tmp = DRIVER + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, "-I", os.path.join(CUDA_HOME, "include"), DRIVER_SRC, "-o", tmp,
          "-L", OUT_DIR, "-lspatialcell", "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart",
          "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")])
    os.replace(tmp, DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
