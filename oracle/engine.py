"""ctypes drivers of the oracle libraries (TEST INFRASTRUCTURE ONLY).

``OracleEngine("port")`` drives oracle/_build/libscport.so (the CPU
restatement), ``OracleEngine("port64")`` its double-precision build
oracle/_build/libscport64.so (the FP64 host oracle); ``OracleEngine("ref")`` drives oracle/_ref/libscref.so (the
reference's own kernels compiled for the host); ``OracleEngine("ref_device")``
drives oracle/_build/librefdev.so, the reference's own kernels compiled for
sm_103a (oracle/_ref/ref_step.cubin) run on the GPU in main.cu's launch
sequence.  All expose the same calls as the product's C ABI, so a test can
run one scenario through all of them.
"""
import ctypes

import numpy as np

from spatial_cell_gb300 import abi

from . import build

_LIBS = {}

_SIGS = {
    "create": (ctypes.c_void_p, [ctypes.POINTER(abi.Config), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_int]),
    "destroy": (None, [ctypes.c_void_p]),
    "load_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int]),
    "run_phase": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "prepare": (ctypes.c_int, [ctypes.c_void_p]),
    "step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "export_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "export_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "get_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(abi.Counters)]),
    "reduce_frame": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
}


def load(kind):
    """Loads (building first if needed) the 'port' or 'ref' library."""
    if kind in _LIBS:
        return _LIBS[kind]
    if kind == "port":
        path, prefix = build.build_port(), "scp_"
    elif kind == "port64":
        path, prefix = build.build_port64(), "scp_"
    elif kind == "ref":
        path, prefix = build.build_ref(), "oref_"
        if path is None:
            raise FileNotFoundError("the reference tree is not present; the reference harness cannot be built")
    elif kind == "ref_device":
        if build.build_ref_cubin() is None:
            raise FileNotFoundError("no oracle/_ref/ref_step.cubin: it is built where the reference tree is present")
        path, prefix = build.build_ref_device(), "refdev_"
    else:
        raise ValueError(kind)
    lib = ctypes.CDLL(path)
    fns = {}
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args if not (kind == "ref_device" and name == "create") else [ctypes.c_char_p] + args
        fns[name] = f
    if kind == "ref_device":
        lib.refdev_last_error.restype = ctypes.c_char_p
        lib.refdev_last_error.argtypes = [ctypes.c_void_p]
        lib.refdev_nonfinite.restype = ctypes.c_int
        lib.refdev_nonfinite.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.refdev_guards.restype = ctypes.c_int
        lib.refdev_guards.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        fns["last_error"] = lib.refdev_last_error
        fns["nonfinite"] = lib.refdev_nonfinite
        fns["guards"] = lib.refdev_guards
    if kind in ("port", "port64"):
        lib.scp_set_threads.argtypes = [ctypes.c_int]
        lib.scp_max_threads.restype = ctypes.c_int
        fns["set_threads"] = lib.scp_set_threads
        fns["max_threads"] = lib.scp_max_threads
    if kind == "ref":
        lib.oref_load_tables.restype = ctypes.c_int
        lib.oref_load_tables.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p] * 4
        lib.oref_load_config.restype = ctypes.c_int
        lib.oref_load_config.argtypes = [ctypes.c_char_p, ctypes.POINTER(abi.Config), ctypes.c_void_p,
                                         ctypes.c_void_p]
        fns["load_tables"] = lib.oref_load_tables
        fns["load_config"] = lib.oref_load_config
    _LIBS[kind] = (lib, fns)
    return _LIBS[kind]


class OracleEngine:
    def __init__(self, kind, cfg, types, rules):
        self.kind = kind
        self.lib, self.f = load(kind)
        self.cfg = cfg
        self.types = np.ascontiguousarray(types, dtype=abi.TYPE_INFO_DTYPE)
        self.rules = np.ascontiguousarray(rules, dtype=abi.RULE_DTYPE)
        args = (ctypes.byref(cfg), abi.ptr(self.types), len(self.types), abi.ptr(self.rules), len(self.rules))
        if kind == "ref_device":
            args = (build.ref_cubin_path().encode(),) + args
        self.h = self.f["create"](*args)
        if not self.h:
            why = self.f["last_error"](None).decode() if kind == "ref_device" else ""
            raise ValueError("oracle rejected the configuration " + why)
        self.n_grid, self.bits, self.cells = abi.grid_dims(cfg)

    def close(self):
        if self.h:
            self.f["destroy"](self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            why = self.f["last_error"](self.h).decode() if self.kind == "ref_device" else ""
            raise RuntimeError(f"{self.kind}: {what} failed ({rc}) {why}")

    def nonfinite(self):
        """Active particles and metabolic items with a non-finite position
        (ref_device only)."""
        out = (ctypes.c_int64 * 2)()
        self._check(self.f["nonfinite"](self.h, out), "nonfinite")
        return int(out[0]), int(out[1])

    def guards(self, cap=64):
        """[(buffer, byte offset)] of the non-zero words in the guard bytes
        around the harness's buffers (ref_device only): stores the reference
        made outside its buffers."""
        names = ctypes.create_string_buffer(32 * cap)
        offs = (ctypes.c_int64 * cap)()
        n = self.f["guards"](self.h, names, 32, offs, cap)
        if n < 0:
            raise RuntimeError("guards failed")
        return [(names.raw[32 * k:32 * (k + 1)].split(b"\0")[0].decode(), int(offs[k])) for k in range(min(n, cap))]

    def load_state(self, particles, metabolic, step=0, next_particle_id=None):
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        m = np.ascontiguousarray(metabolic, abi.METABOLIC_DTYPE)
        if next_particle_id is None:
            next_particle_id = len(p)
        self._check(self.f["load_state"](self.h, abi.ptr(p), len(p), abi.ptr(m), len(m), step, next_particle_id),
                    "load_state")

    def run_phase(self, phase, arg=0):
        self._check(self.f["run_phase"](self.h, phase, arg), f"phase {phase}")

    def prepare(self):
        self._check(self.f["prepare"](self.h), "prepare")

    def step(self, n=1):
        self._check(self.f["step"](self.h, n), "step")

    def export_state(self):
        p = np.zeros(self.cfg.num_particles, abi.PARTICLE_DTYPE)
        m = np.zeros(self.cfg.num_metabolic_particles, abi.METABOLIC_DTYPE)
        self._check(self.f["export_state"](self.h, abi.ptr(p), abi.ptr(m)), "export_state")
        return p, m

    def export_grid(self, which):
        r = np.zeros(self.cells * 2, np.uint32)
        cap = self.cfg.num_metabolic_particles if which else self.cfg.num_particles
        perm = np.zeros(max(cap, 1), np.uint32)
        self._check(self.f["export_grid"](self.h, which, abi.ptr(r), abi.ptr(perm)), "export_grid")
        return r, perm[:cap]

    def counters(self):
        c = abi.Counters()
        self._check(self.f["get_counters"](self.h, ctypes.byref(c)), "get_counters")
        return c

    def reduce_frame(self):
        rp = np.zeros(self.cfg.num_particles, abi.REDUCED_DTYPE)
        rm = np.zeros(self.cfg.num_metabolic_particles, abi.REDUCED_METABOLIC_DTYPE)
        self._check(self.f["reduce_frame"](self.h, abi.ptr(rp), abi.ptr(rm)), "reduce_frame")
        return rp, rm


def set_threads(n):
    lib, f = load("port")
    f["set_threads"](n)


def max_threads():
    lib, f = load("port")
    return f["max_threads"]()


def generate_uniform(n, nm, kinds, fractions, types, box, species, seed):
    """The device scene generator's records built by the CPU oracle
    (spatial_cell_gb300/csrc/sc_gen.h): (particles, metabolic) arrays."""
    lib = ctypes.CDLL(build.build_port())
    f = lib.scp_generate_uniform
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                  ctypes.c_int32, ctypes.c_float, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    k = np.ascontiguousarray(kinds, np.int32)
    fr = np.ascontiguousarray(fractions, np.float32)
    t = np.ascontiguousarray(types, abi.TYPE_INFO_DTYPE)
    p = np.zeros(max(n, 1), abi.PARTICLE_DTYPE)
    m = np.zeros(max(nm, 1), abi.METABOLIC_DTYPE)
    rc = f(n, nm, k.ctypes.data, fr.ctypes.data, len(k), t.ctypes.data, len(t), box, species, seed, p.ctypes.data,
           m.ctypes.data)
    if rc != 0:
        raise ValueError("bad mix")
    return p[:n], m[:nm]


def generate_scene(groups, nm, types, box, species, seed):
    """The structured scene generator's records built by the CPU oracle
    (spatial_cell_gb300/csrc/sc_gen.h): (particles, metabolic) arrays."""
    lib = ctypes.CDLL(build.build_port())
    f = lib.scp_generate_scene
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_float,
                  ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    g = np.ascontiguousarray(np.concatenate([np.atleast_1d(x) for x in groups]), abi.SCENE_GROUP_DTYPE)
    t = np.ascontiguousarray(types, abi.TYPE_INFO_DTYPE)
    n = f(g.ctypes.data, len(g), nm, t.ctypes.data, len(t), box, species, seed, None, None)
    if n < 0:
        raise ValueError("invalid scene groups")
    p = np.zeros(max(n, 1), abi.PARTICLE_DTYPE)
    m = np.zeros(max(nm, 1), abi.METABOLIC_DTYPE)
    f(g.ctypes.data, len(g), nm, t.ctypes.data, len(t), box, species, seed, p.ctypes.data, m.ctypes.data)
    return p[:n], m[:nm]
