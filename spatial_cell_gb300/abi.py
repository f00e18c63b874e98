"""Byte layouts of the C ABI (include/spatialcell.h) as numpy dtypes / ctypes.

The particle records are the reference's structs byte for byte
(spatial_cell_sim/src/types.cuh:167-300): a 256-byte ``Particle``, a 304-byte
``MetabolicParticle`` (NUM_METABOLITES = 10), the 36/44-byte reduced frame
records of frames.dat, the 8-byte ``MinimalParticleTypeInfo`` and the 96-byte
``ParticleInteractionInfo`` rule.
"""
import ctypes

import numpy as np

MAX_ACTIVE_INTERACTIONS = 8
AOS_NUM_METABOLITES = 10
REDUCED_NUM_METABOLITES = 4
PARTICLE_FLAG_ACTIVE = 1
INTERACTION_TYPE_CHAIN = 1
INTERACTION_GROUP_FORWARD = 10
INTERACTION_GROUP_BACKWARD = 11
PARTICLE_TYPE_LIPID = 0
PARTICLE_TYPE_METABOLIC = 1000
HYDROPHYLIC, HYDROPHOBIC, POLAR = 0, 1, 2

_P_NAMES = ["id", "type", "flags", "state", "last_state_change_step", "radius", "hydrophobic", "pos", "rot",
            "velocity", "pos_noise", "angular_velocity", "angular_noise", "n_active_interactions",
            "interactions", "scheduled_polymerization", "debug_vector"]
_P_FORMATS = ["<i4", "<i4", "<i4", "i1", "<i4", "<f4", "i1", ("<f4", 3), ("<f4", 4), ("<f4", 3), ("<f4", 3),
              ("<f4", 4), ("<f4", 4), "<i4", ("<i4", (MAX_ACTIVE_INTERACTIONS, 3)), "<i4", ("<f4", 4)]
_P_OFFSETS = [0, 4, 8, 12, 16, 20, 24, 28, 48, 64, 76, 96, 112, 128, 132, 228, 240]

PARTICLE_DTYPE = np.dtype({"names": _P_NAMES, "formats": _P_FORMATS, "offsets": _P_OFFSETS, "itemsize": 256})
METABOLIC_DTYPE = np.dtype({"names": _P_NAMES + ["metabolites"],
                            "formats": _P_FORMATS + [("<f4", AOS_NUM_METABOLITES)],
                            "offsets": _P_OFFSETS + [256], "itemsize": 304})
REDUCED_DTYPE = np.dtype({"names": ["id", "type", "flags", "radius", "pos", "rot", "debug_vector"],
                          "formats": ["<i4", "<i4", "<i4", "<u2", ("<u2", 3), ("<u2", 4), ("<u2", 4)],
                          "offsets": [0, 4, 8, 12, 14, 20, 28], "itemsize": 36})
REDUCED_METABOLIC_DTYPE = np.dtype({"names": ["id", "type", "flags", "radius", "pos", "rot", "debug_vector",
                                              "metabolites"],
                                    "formats": ["<i4", "<i4", "<i4", "<u2", ("<u2", 3), ("<u2", 4), ("<u2", 4),
                                                ("<u2", REDUCED_NUM_METABOLITES)],
                                    "offsets": [0, 4, 8, 12, 14, 20, 28, 36], "itemsize": 44})
TYPE_INFO_DTYPE = np.dtype({"names": ["radius", "hydrophobic"], "formats": ["<f4", "i1"], "offsets": [0, 4],
                            "itemsize": 8})
RULE_DTYPE = np.dtype({
    "names": ["id", "group", "first_partner_type", "first_partner_state", "second_partner_type",
              "second_partner_state", "propagate_state", "set_state", "wait_for_state", "wait_for_alignment",
              "only_via_transition", "transition_to", "polymerize", "break_after_transition", "use_probability",
              "relative_orientation", "orientation_alignment_threshold", "relative_position",
              "position_alignment_threshold", "probability"],
    "formats": ["<i4", "<i4", "<i4", "i1", "<i4", "i1", "u1", "u1", "u1", "u1", "u1", "<i4", "<i4", "u1", "u1",
                ("<f4", 4), "<f4", ("<f4", 3), "<f4", "<f4"],
    "offsets": [0, 4, 8, 12, 16, 20, 21, 22, 23, 24, 25, 28, 32, 36, 37, 48, 64, 68, 80, 84],
    "itemsize": 96})

# The fields of the reference's ParticleInteractionInfo (the extension fields
# sit in its padding, which the reference leaves unset).
RULE_EXTENSION_FIELDS = ("use_probability", "probability")
RULE_REFERENCE_FIELDS = [n for n in RULE_DTYPE.names if n not in RULE_EXTENSION_FIELDS]

# sc_scene_group (include/spatialcell.h)
SCENE_UNIFORM_BOX = 0
SCENE_UNIFORM_BALL = 1
SCENE_SPHERE_SHELL = 2
SCENE_FIBONACCI_SHELL = 3
SCENE_COMPLEXES = 4
SCENE_WRAPPED_CHAINS = 5
SCENE_MAX_UNIT = 64
SCENE_GROUP_DTYPE = np.dtype({
    "names": ["kind", "count", "unit", "nkinds", "kinds", "fractions", "center", "radius", "spacing", "rot",
              "link_type"],
    "formats": ["<i4", "<i4", "<i4", "<i4", ("<i4", 4), ("<f4", 4), ("<f4", 3), "<f4", "<f4", ("<f4", 4), "<i4"],
    "offsets": [0, 4, 8, 12, 16, 32, 48, 60, 64, 68, 84],
    "itemsize": 88})


def scene_group(kind, count, kinds, fractions=None, center=(0.0, 0.0, 0.0), radius=0.0, unit=1, spacing=0.0,
                rot=(0.0, 0.0, 0.0, 1.0), link_type=1):
    """One sc_scene_group record."""
    g = np.zeros(1, SCENE_GROUP_DTYPE)
    kinds = list(kinds)
    fractions = [1.0] * len(kinds) if fractions is None else list(fractions)
    g["kind"] = kind
    g["count"] = count
    g["unit"] = unit
    g["nkinds"] = len(kinds)
    g["kinds"][0, :len(kinds)] = kinds
    g["fractions"][0, :len(fractions)] = fractions
    g["center"] = center
    g["radius"] = radius
    g["spacing"] = spacing
    g["rot"] = rot
    g["link_type"] = link_type
    return g


def scene_particles(groups):
    """Particles a list of scene groups generates."""
    compound = (SCENE_COMPLEXES, SCENE_WRAPPED_CHAINS)
    g = np.concatenate([np.atleast_1d(x) for x in groups]) if len(groups) else np.zeros(0, SCENE_GROUP_DTYPE)
    per = np.where(np.isin(g["kind"], compound), g["unit"], 1).astype(np.int64)
    return int((g["count"].astype(np.int64) * per).sum())


# sc_phase (include/spatialcell.h)
PHASE_SORT_PARTICLES = 0
PHASE_SORT_METABOLIC = 1
PHASE_MOVE_BROWNIAN = 2
PHASE_MOVE_BROWNIAN_METAB = 3
PHASE_COORDINATE_NOISE = 4
PHASE_APPLY_NOISE = 5
PHASE_RELAX = 6
PHASE_RELAX_METAB = 7
PHASE_RELAX_PARTNERS = 8
PHASE_APPLY_VELOCITIES = 9
PHASE_COMPLEXIFY = 10
PHASE_TRANSITION = 11
PHASE_POLYMERIZE = 12
PHASE_DIFFUSE = 13
PHASE_REMOVE_INTERFERING = 14
PHASE_END_STEP = 15
PHASE_PROPAGATE_STATE = 16


class Config(ctypes.Structure):
    """sc_config: the 17 config.json keys plus extension keys."""
    _fields_ = [
        ("num_particles", ctypes.c_int32),
        ("num_metabolic_particles", ctypes.c_int32),
        ("steps", ctypes.c_int32),
        ("sim_size", ctypes.c_float),
        ("max_interaction_distance", ctypes.c_float),
        ("max_diffusion_distance", ctypes.c_float),
        ("grid_cell_size", ctypes.c_float),
        ("movement_noise_scale", ctypes.c_float),
        ("rotation_noise_scale", ctypes.c_float),
        ("metabolite_movement_noise_scale", ctypes.c_float),
        ("velocity_decay", ctypes.c_float),
        ("angular_velocity_decay", ctypes.c_float),
        ("noise_coordination_steps", ctypes.c_int32),
        ("relaxation_steps", ctypes.c_int32),
        ("metabolite_diffusion_steps", ctypes.c_int32),
        ("persist_every_nth_frame", ctypes.c_int32),
        ("report_every_nth_frame", ctypes.c_int32),
        ("num_metabolites", ctypes.c_int32),
        ("periodic", ctypes.c_int32),
        ("walls", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("graphs", ctypes.c_int32),
        ("class_streams", ctypes.c_int32),
        ("tiles", ctypes.c_int32),
        ("pair_list_limit", ctypes.c_int32),
        ("pool_per_item", ctypes.c_int32),
        ("pair_claim", ctypes.c_int32),
        ("rule_probabilities", ctypes.c_int32),
        ("metabolic_pairs", ctypes.c_int32),
        ("propagate_state", ctypes.c_int32),
        ("_reserved", ctypes.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("_")}


class Replica(ctypes.Structure):
    """sc_replica: one replica cell of a batched sim."""
    _fields_ = [
        ("num_particles", ctypes.c_int32),
        ("num_metabolic_particles", ctypes.c_int32),
        ("sim_size", ctypes.c_float),
        ("_pad", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


class Counters(ctypes.Structure):
    _fields_ = [
        ("n_active_particles", ctypes.c_int32),
        ("n_active_metabolic_particles", ctypes.c_int32),
        ("next_particle_id", ctypes.c_int32),
        ("step", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int64),
        ("device_error", ctypes.c_int32),
        ("_reserved", ctypes.c_int32),
    ]


class Observables(ctypes.Structure):
    _fields_ = [
        ("msd", ctypes.c_double * 2),
        ("msd_items", ctypes.c_int64 * 2),
        ("mean_v2", ctypes.c_double * 2),
        ("active", ctypes.c_int64 * 2),
        ("bond_slots", ctypes.c_int64),
        ("metabolites", ctypes.c_double * AOS_NUM_METABOLITES),
    ]


assert ctypes.sizeof(Config) == 128
assert ctypes.sizeof(Counters) == 32
assert ctypes.sizeof(Replica) == 24

# Reference defaults (spatial_cell_sim/config.json) and extension defaults.
DEFAULT_CONFIG = dict(num_particles=65536, num_metabolic_particles=65536, steps=401, sim_size=400.0,
                      max_interaction_distance=8.0, max_diffusion_distance=10.0, grid_cell_size=10.0,
                      movement_noise_scale=0.7, rotation_noise_scale=0.05, metabolite_movement_noise_scale=1.5,
                      velocity_decay=0.7, angular_velocity_decay=0.7, noise_coordination_steps=16,
                      relaxation_steps=32, metabolite_diffusion_steps=8, persist_every_nth_frame=1,
                      report_every_nth_frame=10, num_metabolites=10, periodic=0, walls=0, seed=42, graphs=1,
                      class_streams=0, tiles=0, pair_list_limit=-1, pool_per_item=-1, pair_claim=0,
                      rule_probabilities=0, metabolic_pairs=1, propagate_state=0)


def make_config(**kw):
    d = dict(DEFAULT_CONFIG)
    unknown = set(kw) - set(d)
    if unknown:
        raise KeyError(f"unknown config keys: {sorted(unknown)}")
    d.update(kw)
    c = Config()
    for k, v in d.items():
        setattr(c, k, v)
    return c


def config_from_bytes(raw):
    """A Config from its bytes; a shorter record written before the
    execution-switch fields existed (the first 88 bytes: the config.json keys,
    num_metabolites, periodic, walls, seed) takes their defaults."""
    raw = bytes(raw)
    c = make_config()
    n = min(len(raw), ctypes.sizeof(Config))
    ctypes.memmove(ctypes.addressof(c), raw, n)
    return c


def grid_dims(cfg):
    """Derived grid of config.cuh:65-74: (cells per axis, bits, total cells)."""
    n = int(np.ceil(np.float32(cfg.sim_size) / np.float32(cfg.grid_cell_size)))
    bits, p2 = 1, 2
    while p2 < n:
        p2 *= 2
        bits += 1
    return p2, bits, p2 ** 3


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)
