"""ctypes binding of libspatialcell.so (include/spatialcell.h).

The library is built in-tree (spatial_cell_gb300/_lib) by
``spatial_cell_gb300.build``.  Loading fails loudly when it is missing: there
is no CPU fallback for any call.
"""
import ctypes
import os

import numpy as np

from . import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libspatialcell.so")

_lib = None

_P = ctypes.c_void_p
_SIGS = {
    "sc_config_defaults": (None, [ctypes.POINTER(abi.Config)]),
    "sc_config_load_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(abi.Config)]),
    "sc_config_grid": (ctypes.c_int, [ctypes.POINTER(abi.Config), ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int32)]),
    "sc_types_load_json": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "sc_rules_load_json": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "sc_create": (ctypes.c_int, [ctypes.POINTER(abi.Config), _P, ctypes.c_int32, _P, ctypes.c_int32,
                                 ctypes.POINTER(_P)]),
    "sc_destroy": (None, [_P]),
    "sc_last_error": (ctypes.c_char_p, [_P]),
    "sc_load_state": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "sc_prepare": (ctypes.c_int, [_P]),
    "sc_step": (ctypes.c_int, [_P, ctypes.c_int32]),
    "sc_run_phase": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "sc_sync": (ctypes.c_int, [_P]),
    "sc_idle": (ctypes.c_int, [_P]),
    "sc_pair_counts": (ctypes.c_int, [_P, _P]),
    "sc_list_overflows": (ctypes.c_int, [_P, _P]),
    "sc_export_state": (ctypes.c_int, [_P, _P, _P]),
    "sc_export_grid": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "sc_get_counters": (ctypes.c_int, [_P, ctypes.POINTER(abi.Counters)]),
    "sc_reduce_frame": (ctypes.c_int, [_P, _P, _P]),
    "sc_reduce_frame_async": (ctypes.c_int64, [_P, _P, _P]),
    "sc_frame_wait": (ctypes.c_int, [_P, ctypes.c_int64]),
    "sc_get_stream": (ctypes.c_void_p, [_P]),
    "sc_device_bytes": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "sc_set_notify": (ctypes.c_int, [_P, ctypes.c_int64]),
    "sc_wait_notices": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int32]),
    "sc_generate_uniform": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, _P, _P, ctypes.c_int32,
                                           ctypes.c_uint64]),
    "sc_generate_scene": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64]),
    "sc_mark_positions": (ctypes.c_int, [_P]),
    "sc_observe": (ctypes.c_int, [_P, ctypes.POINTER(abi.Observables)]),
    "sc_pair_histogram": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_int32, _P]),
    "sc_checkpoint_write": (ctypes.c_int, [_P, _P]),
    "sc_checkpoint_read": (ctypes.c_int, [_P, _P]),
    "sc_frames_write_header": (ctypes.c_int, [_P, ctypes.POINTER(abi.Config)]),
    "sc_frames_write_frame": (ctypes.c_int, [_P, ctypes.POINTER(abi.Config), _P, _P]),
    "sc_sort_cells_static": (ctypes.c_int, [ctypes.POINTER(abi.Config), _P, _P, ctypes.c_int32, _P, _P, _P]),
    "sc_create_batch": (ctypes.c_int, [ctypes.POINTER(abi.Config), _P, ctypes.c_int32, _P, ctypes.c_int32, _P,
                                       ctypes.c_int32, ctypes.POINTER(_P)]),
    "sc_load_batch": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int32]),
    "sc_export_replica": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "sc_generate_batch": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int32, _P]),
    "sc_generate_scene_batch": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int32, _P]),
}

# Every symbol include/spatialcell.h declares.
EXPORTED = tuple(_SIGS)


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; build it with `python -m spatial_cell_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class ScError(RuntimeError):
    pass


class _cfile:
    """A C FILE* for the ABI's file functions."""

    def __init__(self, path, mode):
        self.libc = ctypes.CDLL(None)
        self.libc.fopen.restype = ctypes.c_void_p
        self.libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        self.libc.fclose.argtypes = [ctypes.c_void_p]
        self.f = self.libc.fopen(str(path).encode(), mode)
        if not self.f:
            raise OSError(f"cannot open {path}")

    def __enter__(self):
        return ctypes.c_void_p(self.f)

    def __exit__(self, *a):
        self.libc.fclose(self.f)


def _check(rc, sim=None, what=""):
    if rc != 0:
        msg = lib().sc_last_error(sim)
        raise ScError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")


def load_config_json(path, base=None):
    c = abi.make_config() if base is None else base
    _check(lib().sc_config_load_json(path.encode(), ctypes.byref(c)), None, "sc_config_load_json")
    return c


def load_types_json(path):
    n = ctypes.c_int32(0)
    _check(lib().sc_types_load_json(path.encode(), None, 0, ctypes.byref(n)), None, "sc_types_load_json")
    out = np.zeros(n.value, abi.TYPE_INFO_DTYPE)
    _check(lib().sc_types_load_json(path.encode(), abi.ptr(out), n.value, ctypes.byref(n)), None, "sc_types_load_json")
    return out


def load_rules_json(path):
    n = ctypes.c_int32(0)
    _check(lib().sc_rules_load_json(path.encode(), None, 0, ctypes.byref(n)), None, "sc_rules_load_json")
    out = np.zeros(n.value, abi.RULE_DTYPE)
    _check(lib().sc_rules_load_json(path.encode(), abi.ptr(out), n.value, ctypes.byref(n)), None, "sc_rules_load_json")
    return out


def wait_notices(cap=1024, timeout_ms=-1):
    """Keys of sims whose stepping finished (sc_wait_notices), in order;
    blocks up to timeout_ms (the GIL is released while it waits)."""
    buf = (ctypes.c_int64 * cap)()
    n = lib().sc_wait_notices(buf, cap, timeout_ms)
    if n < 0:
        _check(n, None, "sc_wait_notices")
    return [int(buf[k]) for k in range(n)]


def grid(cfg):
    n, b = ctypes.c_int32(0), ctypes.c_int32(0)
    _check(lib().sc_config_grid(ctypes.byref(cfg), ctypes.byref(n), ctypes.byref(b)), None, "sc_config_grid")
    return n.value, b.value


class Simulation:
    """One simulation on the current CUDA device (include/spatialcell.h)."""

    def __init__(self, cfg, types, rules, replicas=None):
        self.L = lib()
        self.cfg = cfg
        self.types = np.ascontiguousarray(types, dtype=abi.TYPE_INFO_DTYPE)
        self.rules = np.ascontiguousarray(rules, dtype=abi.RULE_DTYPE)
        h = ctypes.c_void_p()
        if replicas is None:
            _check(self.L.sc_create(ctypes.byref(cfg), abi.ptr(self.types), len(self.types), abi.ptr(self.rules),
                                    len(self.rules), ctypes.byref(h)), None, "sc_create")
            self.n_grid, self.bits, self.cells = abi.grid_dims(cfg)
        else:
            self.replicas = (abi.Replica * len(replicas))(*replicas)
            _check(self.L.sc_create_batch(ctypes.byref(cfg), self.replicas, len(replicas), abi.ptr(self.types),
                                          len(self.types), abi.ptr(self.rules), len(self.rules), ctypes.byref(h)),
                   None, "sc_create_batch")
            # the batch's capacities and key space
            self.cfg = abi.config_from_bytes(bytes(cfg))
            self.cfg.num_particles = sum(r.num_particles for r in replicas)
            self.cfg.num_metabolic_particles = sum(r.num_metabolic_particles for r in replicas)
            self.cells = sum(abi.grid_dims(abi.make_config(sim_size=r.sim_size,
                                                           grid_cell_size=cfg.grid_cell_size))[2] for r in replicas)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.sc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load_state(self, particles, metabolic, step=0, next_particle_id=None):
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        m = np.ascontiguousarray(metabolic, abi.METABOLIC_DTYPE)
        if next_particle_id is None:
            next_particle_id = len(p)
        _check(self.L.sc_load_state(self.h, abi.ptr(p), len(p), abi.ptr(m), len(m), step, next_particle_id), self.h,
               "sc_load_state")

    def load_batch(self, states, step=0):
        """Loads a batched sim: states[r] = (particles, metabolic) of replica r."""
        n = np.array([len(x[0]) for x in states], np.int32)
        nm = np.array([len(x[1]) for x in states], np.int32)
        # filled slice by slice: np.concatenate would drop the records' padded layout
        p = np.zeros(int(n.sum()), abi.PARTICLE_DTYPE)
        m = np.zeros(int(nm.sum()), abi.METABOLIC_DTYPE)
        o = om = 0
        for (pp, mm), k, km in zip(states, n, nm):
            p[o:o + k] = pp
            m[om:om + km] = mm
            o += k
            om += km
        _check(self.L.sc_load_batch(self.h, abi.ptr(p), abi.ptr(n), abi.ptr(m), abi.ptr(nm), step), self.h,
               "sc_load_batch")

    def generate_batch(self, n, nm, kinds, fractions, seeds):
        """Fills a batched sim on the device (sc_generate_batch): replica r gets
        n[r] particles of the kinds with weights fractions[r] and nm[r]
        metabolic particles, seeded by seeds[r]."""
        n = np.ascontiguousarray(n, np.int32)
        nm = np.ascontiguousarray(nm, np.int32)
        k = np.ascontiguousarray(kinds, np.int32)
        f = np.ascontiguousarray(fractions, np.float32).reshape(len(n), len(k))
        sd = np.ascontiguousarray(seeds, np.uint64)
        _check(self.L.sc_generate_batch(self.h, abi.ptr(n), abi.ptr(nm), abi.ptr(k), abi.ptr(f), len(k), abi.ptr(sd)),
               self.h, "sc_generate_batch")

    def export_replica(self, r):
        """Replica r's records (sc_export_replica), arrays of its capacities."""
        q = self.replicas[r]
        p = np.zeros(q.num_particles, abi.PARTICLE_DTYPE)
        m = np.zeros(q.num_metabolic_particles, abi.METABOLIC_DTYPE)
        _check(self.L.sc_export_replica(self.h, r, abi.ptr(p), abi.ptr(m)), self.h, "sc_export_replica")
        return p, m

    def load_state_ptr(self, p_ptr, n, m_ptr, nm, step=0, next_particle_id=0):
        """Loads from raw host pointers (e.g. pinned buffers)."""
        _check(self.L.sc_load_state(self.h, p_ptr, n, m_ptr, nm, step, next_particle_id), self.h, "sc_load_state")

    def generate_uniform(self, n, nm, kinds, fractions, seed):
        """Fills the sim on the device (sc_generate_uniform): n particles of the
        given kinds / weights and nm metabolic particles, uniform in the box."""
        k = np.ascontiguousarray(kinds, np.int32)
        f = np.ascontiguousarray(fractions, np.float32)
        _check(self.L.sc_generate_uniform(self.h, n, nm, abi.ptr(k), abi.ptr(f), len(k), seed), self.h,
               "sc_generate_uniform")

    def generate_scene(self, groups, nm, seed):
        """Fills the sim on the device (sc_generate_scene): the particles of
        the scene groups (abi.SCENE_GROUP_DTYPE records), one group after
        another, and nm metabolic particles uniform in the box."""
        g = np.ascontiguousarray(np.concatenate([np.atleast_1d(x) for x in groups]) if len(groups) else
                                 np.zeros(0, abi.SCENE_GROUP_DTYPE), abi.SCENE_GROUP_DTYPE)
        _check(self.L.sc_generate_scene(self.h, abi.ptr(g) if len(g) else None, len(g), nm, seed), self.h,
               "sc_generate_scene")

    def generate_scene_batch(self, groups, nm, seeds):
        """Fills a batched sim on the device (sc_generate_scene_batch): every
        replica r gets the scene groups' particles and nm metabolic particles,
        seeded by seeds[r]."""
        g = np.ascontiguousarray(np.concatenate([np.atleast_1d(x) for x in groups]) if len(groups) else
                                 np.zeros(0, abi.SCENE_GROUP_DTYPE), abi.SCENE_GROUP_DTYPE)
        sd = np.ascontiguousarray(seeds, np.uint64)
        _check(self.L.sc_generate_scene_batch(self.h, abi.ptr(g) if len(g) else None, len(g), nm, abi.ptr(sd)),
               self.h, "sc_generate_scene_batch")

    def prepare(self):
        _check(self.L.sc_prepare(self.h), self.h, "sc_prepare")

    def step(self, n=1):
        _check(self.L.sc_step(self.h, n), self.h, "sc_step")

    def pair_counts(self):
        """Pairs in the current lists: (particle, metabolic, lipid-metabolic, diffusion), -1 if not built."""
        out = np.zeros(4, np.int64)
        _check(self.L.sc_pair_counts(self.h, abi.ptr(out)), self.h, "sc_pair_counts")
        return tuple(int(x) for x in out)

    def mark_positions(self):
        """Records the current positions as the origin of the MSD (sc_mark_positions)."""
        _check(self.L.sc_mark_positions(self.h), self.h, "sc_mark_positions")

    def observe(self):
        """FP64 observables (sc_observe) as a dict: msd, msd_items, mean_v2, active
        (each a (particles, metabolic) pair), bond_slots, metabolites."""
        o = abi.Observables()
        _check(self.L.sc_observe(self.h, ctypes.byref(o)), self.h, "sc_observe")
        return {"msd": tuple(o.msd), "msd_items": tuple(o.msd_items), "mean_v2": tuple(o.mean_v2),
                "active": tuple(o.active), "bond_slots": int(o.bond_slots),
                "metabolites": tuple(o.metabolites)}

    def pair_histogram(self, type_a, type_b, r_max, n_bins):
        """Distance histogram of ordered particle pairs (sc_pair_histogram)."""
        out = np.zeros(n_bins, np.uint64)
        _check(self.L.sc_pair_histogram(self.h, type_a, type_b, r_max, n_bins, abi.ptr(out)), self.h,
               "sc_pair_histogram")
        return out

    def list_overflows(self):
        """Items whose list overflowed, per list as pair_counts; -1 if not built."""
        out = np.zeros(4, np.int64)
        _check(self.L.sc_list_overflows(self.h, abi.ptr(out)), self.h, "sc_list_overflows")
        return tuple(int(x) for x in out)

    def idle(self):
        """True when all work enqueued on this sim has finished (does not wait)."""
        rc = self.L.sc_idle(self.h)
        if rc < 0:
            _check(rc, self.h, "sc_idle")
        return rc == 1

    def run_phase(self, phase, arg=0):
        _check(self.L.sc_run_phase(self.h, phase, arg), self.h, f"sc_run_phase({phase})")

    def sync(self):
        _check(self.L.sc_sync(self.h), self.h, "sc_sync")

    def export_state(self):
        p = np.zeros(self.cfg.num_particles, abi.PARTICLE_DTYPE)
        m = np.zeros(self.cfg.num_metabolic_particles, abi.METABOLIC_DTYPE)
        _check(self.L.sc_export_state(self.h, abi.ptr(p), abi.ptr(m)), self.h, "sc_export_state")
        return p, m

    def export_grid(self, which):
        r = np.zeros(self.cells * 2, np.uint32)
        cap = self.cfg.num_metabolic_particles if which else self.cfg.num_particles
        perm = np.zeros(max(cap, 1), np.uint32)
        _check(self.L.sc_export_grid(self.h, which, abi.ptr(r), abi.ptr(perm)), self.h, "sc_export_grid")
        return r, perm[:cap]

    def set_notify(self, key):
        """Queue `key` each time this sim's sc_step work finishes (see wait_notices)."""
        _check(self.L.sc_set_notify(self.h, key), self.h, "sc_set_notify")

    def device_bytes(self):
        """Device memory the sim holds now (sc_device_bytes)."""
        b = ctypes.c_int64(0)
        _check(self.L.sc_device_bytes(self.h, ctypes.byref(b)), self.h, "sc_device_bytes")
        return b.value

    def stream_handle(self):
        """The sim's cudaStream_t as an integer."""
        return self.L.sc_get_stream(self.h)

    def counters(self):
        c = abi.Counters()
        _check(self.L.sc_get_counters(self.h, ctypes.byref(c)), self.h, "sc_get_counters")
        return c

    def reduce_frame(self, out_p=None, out_m=None):
        rp = np.zeros(self.cfg.num_particles, abi.REDUCED_DTYPE) if out_p is None else out_p
        rm = np.zeros(self.cfg.num_metabolic_particles, abi.REDUCED_METABOLIC_DTYPE) if out_m is None else out_m
        _check(self.L.sc_reduce_frame(self.h, abi.ptr(rp), abi.ptr(rm)), self.h, "sc_reduce_frame")
        return rp, rm

    def reduce_frame_ptr(self, p_ptr, m_ptr):
        _check(self.L.sc_reduce_frame(self.h, p_ptr, m_ptr), self.h, "sc_reduce_frame")

    def reduce_frame_async_ptr(self, p_ptr, m_ptr):
        """Streams the current frame into (pinned) host buffers; returns its ticket."""
        t = self.L.sc_reduce_frame_async(self.h, p_ptr, m_ptr)
        if t < 0:
            _check(int(t), self.h, "sc_reduce_frame_async")
        return t

    def frame_wait(self, ticket):
        _check(self.L.sc_frame_wait(self.h, ticket), self.h, "sc_frame_wait")

    def checkpoint(self, path):
        """Writes the whole state to `path` (sc_checkpoint_write)."""
        with _cfile(path, b"wb") as f:
            _check(self.L.sc_checkpoint_write(self.h, f), self.h, "sc_checkpoint_write")

    def resume(self, path):
        """Loads a checkpoint; the next step continues the saved run."""
        with _cfile(path, b"rb") as f:
            _check(self.L.sc_checkpoint_read(self.h, f), self.h, "sc_checkpoint_read")
