"""The periodic box extension, on the oracle.

``sc_config.periodic = 1`` is an extension with no counterpart in the
reference: the reference clamps positions to [0, simSize]
(spatial_cell_sim/src/dynamics.cuh, applyVelocities) and clamps cell indices
at the walls (spatial_cell_sim/src/grid_geometry.cuh).  At the measured
workloads' densities the clamp piles particles into the box's corners, where
coincident particles normalise a zero vector and the resulting NaNs spread.
In a periodic box positions wrap, neighbour cells wrap over the cells the box
spans and every pair distance uses the nearest image.  These tests check the
oracle's periodic mode on properties it must have; the CUDA path is compared
with it bit for bit in tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes


def _workload(n, nm, box, seed, periodic, steps_cfg=None):
    cfg = scenes.workload_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box,
                                 num_metabolites=10, seed=seed, periodic=periodic, **(steps_cfg or {}))
    rng = np.random.default_rng(seed)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, box, types)
    m = scenes.uniform_metabolic(rng, nm, box, types, 10)
    return cfg, types, rules, p, m


def _engine(cfg, types, rules, p, m):
    from oracle.engine import OracleEngine
    e = OracleEngine("port", cfg, types, rules)
    e.load_state(p, m, step=0, next_particle_id=len(p))
    return e


def test_positions_wrap_and_stay_finite():
    cfg, types, rules, p, m = _workload(3000, 6000, 70.0, 11, periodic=1,
                                        steps_cfg=dict(relaxation_steps=12, noise_coordination_steps=6))
    e = _engine(cfg, types, rules, p, m)
    e.prepare()
    e.step(3)
    gp, gm = e.export_state()
    act = (gp["flags"] & abi.PARTICLE_FLAG_ACTIVE) != 0
    for recs, name in ((gp[act], "particles"), (gm[(gm["flags"] & 1) != 0], "metabolic")):
        pos = recs["pos"]
        assert np.isfinite(pos).all(), f"{name}: non-finite positions"
        assert (pos >= 0).all() and (pos < cfg.sim_size).all(), f"{name}: positions outside [0, L)"
        assert np.isfinite(recs["velocity"]).all(), f"{name}: non-finite velocities"


def test_periodic_equals_walls_away_from_the_boundary():
    """A cluster far from every face never sees an image or a wrapped cell,
    so a periodic box and the reference walls give the same bytes."""
    rng = np.random.default_rng(4)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    box, n, nm = 96.0, 600, 900
    p = scenes.uniform_particles(rng, n, 24.0, types)
    m = scenes.uniform_metabolic(rng, nm, 24.0, types, 10)
    p["pos"] += np.float32(36.0)
    m["pos"] += np.float32(36.0)
    out = []
    for periodic in (0, 1):
        cfg = scenes.workload_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box,
                                     num_metabolites=10, seed=9, periodic=periodic, relaxation_steps=8,
                                     noise_coordination_steps=4)
        e = _engine(cfg, types, rules, p, m)
        e.prepare()
        e.step(2)
        out.append(e.export_state())
    assert out[0][0].tobytes() == out[1][0].tobytes()
    assert out[0][1].tobytes() == out[1][1].tobytes()


def test_pair_across_the_face_interacts_through_the_image():
    """Two lipids 1 unit apart across the x face attract/repel as neighbours in
    a periodic box; with walls they are a whole box apart and do not."""
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    box = 60.0
    p = scenes.blank_particles(2)
    p["id"] = [0, 1]
    p["type"] = scenes.LIPID
    p["radius"] = types["radius"][scenes.LIPID]
    p["pos"] = [[0.4, 30.0, 30.0], [box - 0.6, 30.0, 30.0]]
    p["rot"] = [[0, 0, 0, 1]] * 2
    p["angular_velocity"] = [[0, 0, 0, 1]] * 2
    m = scenes.uniform_metabolic(np.random.default_rng(0), 4, 8.0, types, 10)
    m["pos"] += np.float32(10.0)
    moved = {}
    for periodic in (0, 1):
        cfg = scenes.workload_config("plain_small", num_particles=8, num_metabolic_particles=8, sim_size=box,
                                     num_metabolites=10, seed=2, periodic=periodic, movement_noise_scale=0.0,
                                     rotation_noise_scale=0.0, relaxation_steps=4)
        e = _engine(cfg, types, rules, p, m)
        e.run_phase(abi.PHASE_SORT_PARTICLES)
        e.run_phase(abi.PHASE_RELAX, 0)
        gp, _ = e.export_state()
        moved[periodic] = np.abs(gp["velocity"]).max()
    assert moved[0] == 0.0
    assert moved[1] > 0.0


def test_pair_across_the_face_of_a_box_not_a_multiple_of_the_cell():
    """A 50 nm box with 6 nm cells is split into 8 equal cells of 6.25 nm (not
    8 of 6 and a 2 nm sliver), so a pair 4 nm apart across the face, one of
    them 3 nm inside it, is in neighbouring cells and collides (radii 2.5)."""
    box = 50.0
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.blank_particles(2)
    p["id"] = [0, 1]
    p["type"] = scenes.TYPE_A
    p["radius"] = types["radius"][scenes.TYPE_A]
    p["pos"] = [[1.0, 20.0, 20.0], [box - 3.0, 20.0, 20.0]]
    p["rot"] = [[0, 0, 0, 1]] * 2
    p["angular_velocity"] = [[0, 0, 0, 1]] * 2
    m = scenes.uniform_metabolic(np.random.default_rng(0), 4, 8.0, types, 10)
    m["pos"] += np.float32(10.0)
    cfg = scenes.workload_config("plain_small", num_particles=8, num_metabolic_particles=8, sim_size=box,
                                 num_metabolites=10, seed=2, periodic=1, movement_noise_scale=0.0,
                                 rotation_noise_scale=0.0, relaxation_steps=4)
    e = _engine(cfg, types, rules, p, m)
    e.run_phase(abi.PHASE_SORT_PARTICLES)
    e.run_phase(abi.PHASE_RELAX, 0)
    gp, _ = e.export_state()
    assert np.abs(gp["velocity"]).max() > 0.0  # 4 nm < 2.5 + 2.5: they overlap and push apart


def test_reflecting_walls_mirror_a_step_past_the_wall():
    """With walls = 1 a step that leaves the box is mirrored back into it
    (the reference clamps it onto the wall instead)."""
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    box = 30.0
    p = scenes.blank_particles(2)
    p["id"] = [0, 1]
    p["type"] = scenes.DUMMY
    p["radius"] = types["radius"][scenes.DUMMY]
    p["pos"] = [[0.5, 15.0, 15.0], [29.0, 15.0, 15.0]]
    p["velocity"] = [[-2.0, 0.0, 0.0], [4.0, 0.0, 0.0]]
    p["rot"] = [[0, 0, 0, 1]] * 2
    p["angular_velocity"] = [[0, 0, 0, 1]] * 2
    m = scenes.uniform_metabolic(np.random.default_rng(0), 4, 8.0, types, 10)
    m["pos"] += np.float32(10.0)
    got = {}
    for walls in (0, 1):
        cfg = scenes.workload_config("plain_small", num_particles=8, num_metabolic_particles=8, sim_size=box,
                                     num_metabolites=10, seed=2, periodic=0, walls=walls)
        e = _engine(cfg, types, rules, p, m)
        e.run_phase(abi.PHASE_APPLY_VELOCITIES)
        gp, _ = e.export_state()
        gp = gp[(gp["flags"] & abi.PARTICLE_FLAG_ACTIVE) != 0]
        got[walls] = gp["pos"][np.argsort(gp["id"])][:, 0]
    # x + 0.45 v: 0.5 - 0.9 = -0.4 and 29 + 1.8 = 30.8
    assert got[0].tolist() == [0.0, 30.0]
    assert np.allclose(got[1], [0.4, 29.2], atol=1e-5)


def test_oracle_rejects_a_box_of_fewer_than_three_cells():
    from oracle.engine import OracleEngine
    cfg = abi.make_config(num_particles=8, num_metabolic_particles=8, sim_size=12.0, grid_cell_size=6.0,
                          periodic=1)
    with pytest.raises(Exception):
        OracleEngine("port", cfg, scenes.baseline_types(), scenes.baseline_rules())
