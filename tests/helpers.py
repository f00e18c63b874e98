"""Comparison helpers of the parity tests."""
import numpy as np

from spatial_cell_gb300 import abi


def _bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype.kind == "f":
        return a.view(np.uint32 if a.dtype.itemsize == 4 else np.uint64)
    return a


def mask_state(p, m, species=abi.AOS_NUM_METABOLITES):
    """Copies with the bytes that carry no state zeroed: interaction slots at
    and beyond n_active_interactions (never read by any kernel) and metabolite
    species at and beyond the simulated count."""
    p = p.copy()
    m = m.copy()
    for arr in (p, m):
        nb = np.clip(arr["n_active_interactions"], 0, abi.MAX_ACTIVE_INTERACTIONS)
        slot = np.arange(abi.MAX_ACTIVE_INTERACTIONS)[None, :]
        arr["interactions"][slot >= nb[:, None]] = 0
    m["metabolites"][:, species:] = 0
    return p, m


def diff_fields(a, b, limit=4):
    """Field-by-field bitwise comparison; returns a list of mismatch lines."""
    out = []
    assert a.dtype == b.dtype and a.shape == b.shape, (a.dtype, b.dtype, a.shape, b.shape)
    for name in a.dtype.names:
        x, y = _bits(a[name]), _bits(b[name])
        ne = (x != y).reshape(len(x), -1).any(axis=1)
        if ne.any():
            idx = np.nonzero(ne)[0]
            out.append(f"{name}: {len(idx)} items differ, first {idx[:limit].tolist()}: "
                       f"{a[name][idx[:2]].tolist()} vs {b[name][idx[:2]].tolist()}")
    return out


def assert_same_state(sa, sb, species=abi.AOS_NUM_METABOLITES, what=""):
    pa, ma = mask_state(*sa, species=species)
    pb, mb = mask_state(*sb, species=species)
    problems = [f"particles {d}" for d in diff_fields(pa, pb)] + [f"metabolic {d}" for d in diff_fields(ma, mb)]
    assert not problems, f"{what}: state differs\n" + "\n".join(problems)


def assert_same_counters(ca, cb, what=""):
    for k in ("n_active_particles", "n_active_metabolic_particles", "next_particle_id", "step"):
        assert getattr(ca, k) == getattr(cb, k), f"{what}: counter {k} {getattr(ca, k)} != {getattr(cb, k)}"


# The launch order of one step (main.cu:347-661) as (phase, arg) pairs.
def step_phases(cfg):
    ph = [(abi.PHASE_SORT_PARTICLES, 0), (abi.PHASE_SORT_METABOLIC, 0), (abi.PHASE_MOVE_BROWNIAN, 0),
          (abi.PHASE_MOVE_BROWNIAN_METAB, 0)]
    ph += [(abi.PHASE_COORDINATE_NOISE, j) for j in range(cfg.noise_coordination_steps)]
    ph += [(abi.PHASE_APPLY_NOISE, 0)]
    for j in range(cfg.relaxation_steps):
        ph.append((abi.PHASE_RELAX, j))
        if j % 2 == 0:
            ph += [(abi.PHASE_RELAX_METAB, j), (abi.PHASE_RELAX_PARTNERS, j)]
    ph += [(abi.PHASE_APPLY_VELOCITIES, 0), (abi.PHASE_COMPLEXIFY, 0), (abi.PHASE_TRANSITION, 0),
           (abi.PHASE_POLYMERIZE, 0)]
    if getattr(cfg, "propagate_state", 0):
        ph += [(abi.PHASE_PROPAGATE_STATE, 0)]
    ph += [(abi.PHASE_DIFFUSE, j) for j in range(cfg.metabolite_diffusion_steps)]
    ph += [(abi.PHASE_END_STEP, 0)]
    return ph
