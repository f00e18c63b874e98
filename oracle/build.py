"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

    python -m oracle.build            # port, plus the reference's builds when
                                      # the reference tree is present

* oracle/_build/libscport.so  <- oracle/scport.cpp (g++, OpenMP)
* oracle/_build/libscport64.so <- oracle/scport64.cpp: the same restatement
                                 in double precision (the FP64 host oracle)
* oracle/_ref/libscref.so     <- oracle/ref_harness.cpp + the reference's
                                 spatial_cell_sim/src/*.cuh read in place,
                                 with oracle/shim first on the include path
                                 (the reference's kernels on the host CPU)
* oracle/_ref/ref_step.cubin  <- oracle/ref_device_kernels.cu + the same
                                 reference headers, with oracle/shim_dev first
                                 (the reference's kernels for sm_103a; built
                                 where the reference tree is, run where the
                                 GPU is)
* oracle/_build/librefdev.so  <- oracle/ref_device.cu (nvcc + the toolkit's
                                 CUB): loads ref_step.cubin and replays the
                                 reference's launch sequence on the GPU

All are built without fused multiply-adds (-ffp-contract=off on the host,
-fmad=false for the device): every floating-point operation is rounded
exactly as written.
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


def port64_path():
    return os.path.join(HERE, "_build", "libscport64.so")


def build_port64(force=False):
    """The FP64 build of the CPU restatement (oracle/scport64.cpp)."""
    out = port64_path()
    srcs = [os.path.join(HERE, "scport64.cpp"), os.path.join(HERE, "scport.cpp"), os.path.join(HERE, "scmath64.h"),
            os.path.join(CSRC, "scmath.h"), os.path.join(CSRC, "sc_gen.h"), os.path.join(INCLUDE, "spatialcell.h")]
    if not force and _newer(out, srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run(["g++", "-std=c++17", "-fPIC", "-shared", "-fopenmp", *FP_FLAGS, "-I", CSRC, "-I", INCLUDE, "-I", HERE,
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


NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def ref_cubin_path():
    return os.path.join(HERE, "_ref", "ref_step.cubin")


def ref_device_path():
    return os.path.join(HERE, "_build", "librefdev.so")


def build_ref_cubin(force=False):
    """Compiles the reference's kernels for sm_103a; None if the reference
    tree is absent (the cubin built where it is present is used as is)."""
    if not reference_available():
        return ref_cubin_path() if os.path.exists(ref_cubin_path()) else None
    out = ref_cubin_path()
    shim = os.path.join(HERE, "shim_dev")
    srcs = [os.path.join(HERE, "ref_device_kernels.cu"), os.path.join(CSRC, "scmath.h"),
            os.path.join(INCLUDE, "spatialcell.h"), os.path.join(HERE, "shim", "json", "json.h")] + \
        [os.path.join(shim, f) for f in os.listdir(shim) if f.endswith(".h")]
    if not force and _newer(out, srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run([NVCC, "-cubin", *ARCH, "-std=c++17", "-O3", "-fmad=false", "-w", "-I", shim, "-I", CSRC, "-I", INCLUDE,
          "-I", REFERENCE_SRC, "-include", "sc_ref_device_prelude.h", srcs[0], "-o", out])
    return out


def build_ref_device(force=False):
    """The GPU harness of the reference's step (needs only the toolkit)."""
    out = ref_device_path()
    srcs = [os.path.join(HERE, "ref_device.cu"), os.path.join(INCLUDE, "spatialcell.h")]
    if not force and _newer(out, srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run([NVCC, "-shared", "-Xcompiler", "-fPIC", "-std=c++17", "-O2", *ARCH, "-I", INCLUDE, srcs[0], "-o", out,
          "-lcuda"])
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_port(force=force))
    print(build_port64(force=force))
    print(build_ref(force=force))
    print(build_ref_cubin(force=force))
    print(build_ref_device(force=force))
