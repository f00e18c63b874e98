"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE ONLY).

    python -m oracle.build            # port, plus the reference harness when
                                      # the reference tree is present

* oracle/_build/libscport.so  <- oracle/scport.cpp (g++, OpenMP)
* oracle/_ref/libscref.so     <- oracle/ref_harness.cpp + the reference's
                                 spatial_cell_sim/src/*.cuh read in place,
                                 with oracle/shim first on the include path

Both are built with -ffp-contract=off so no multiply-add is fused (the
sm_103a build uses -fmad=false for the same reason): every floating-point
operation is rounded exactly as written.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE_SRC = os.environ.get("SC_REFERENCE_SRC", "/root/reference/spatial_cell_sim/src")
CSRC = os.path.join(ROOT, "spatial_cell_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")
FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fno-finite-math-only"]


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def port_path():
    return os.path.join(HERE, "_build", "libscport.so")


def ref_path():
    return os.path.join(HERE, "_ref", "libscref.so")


def build_port(force=False):
    out = port_path()
    srcs = [os.path.join(HERE, "scport.cpp"), os.path.join(CSRC, "scmath.h"), os.path.join(CSRC, "sc_gen.h"),
            os.path.join(INCLUDE, "spatialcell.h")]
    if not force and _newer(out, srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run(["g++", "-std=c++17", "-fPIC", "-shared", "-fopenmp", *FP_FLAGS, "-I", CSRC, "-I", INCLUDE,
          srcs[0], "-o", out])
    return out


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_SRC, "dynamics.cuh"))


def build_ref(force=False):
    """Compiles the reference's kernels for the host; None if the reference
    tree is absent."""
    if not reference_available():
        return None
    out = ref_path()
    shim = os.path.join(HERE, "shim")
    srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(CSRC, "scmath.h"), os.path.join(CSRC, "sc_json.hpp"),
            os.path.join(INCLUDE, "spatialcell.h")] + [os.path.join(shim, f) for f in os.listdir(shim)
                                                        if f.endswith(".h")]
    if not force and _newer(out, srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run(["g++", "-std=c++17", "-fPIC", "-shared", "-w", *FP_FLAGS, "-I", shim, "-I", CSRC, "-I", INCLUDE,
          "-I", REFERENCE_SRC, "-include", "sc_ref_prelude.h", srcs[0], "-o", out])
    return out


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
