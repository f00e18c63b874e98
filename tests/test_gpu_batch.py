"""Batched sims: many replica cells stepped by one launch per phase.

A batch (sc_create_batch) holds the replicas' items side by side, sorts
them in one key space (the replica above the cell), and runs every kernel
once over all of them, each item with its replica's box, cells and noise
key.  Every replica must evolve exactly as a sim of its own with the same
config, box, capacities and seed -- and as the CPU oracle -- bit for bit.
"""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_state


def _replicas(count, seed, periodic=1, n_lo=600, n_hi=5000, claim=1):
    reps = scenes.batch_replicas(count, seed=seed, n_lo=n_lo, n_hi=n_hi)
    out = []
    for cfg, types, rules, p, m in reps:
        cfg.periodic = periodic
        cfg.pair_claim = claim
        cfg.noise_coordination_steps, cfg.relaxation_steps, cfg.metabolite_diffusion_steps = 4, 6, 3
        out.append((cfg, types, rules, p, m))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("periodic,claim", [(1, 1), (0, 0)])
def test_each_replica_equals_its_own_sim_and_the_oracle(product, periodic, claim):
    from oracle.engine import OracleEngine
    reps = _replicas(5, seed=11, periodic=periodic, claim=claim)
    cfg, replicas = scenes.batch_of(reps)
    types, rules = reps[0][1], reps[0][2]
    batch = product.Simulation(cfg, types, rules, replicas=replicas)
    batch.load_batch([(p, m) for _, _, _, p, m in reps])
    batch.prepare()
    batch.step(2)
    for r, (c, t, ru, p, m) in enumerate(reps):
        got = batch.export_replica(r)
        solo = product.Simulation(c, t, ru)
        cpu = OracleEngine("port", c, t, ru)
        for e in (solo, cpu):
            e.load_state(p, m)
            e.prepare()
            e.step(2)
        assert_same_state(got, solo.export_state(), species=c.num_metabolites, what=f"replica {r} vs its own sim")
        assert_same_state(got, cpu.export_state(), species=c.num_metabolites, what=f"replica {r} vs the oracle")
        solo.close()
        cpu.close()
    assert batch.counters().n_active_particles == sum(len(x[3]) for x in reps)
    batch.close()


@pytest.mark.gpu
def test_batch_graph_steps_equal_direct_steps(product):
    reps = _replicas(4, seed=12)
    cfg, replicas = scenes.batch_of(reps)
    out = []
    for graphs in (1, 0):
        c = abi.config_from_bytes(bytes(cfg))
        c.graphs = graphs
        b = product.Simulation(c, reps[0][1], reps[0][2], replicas=replicas)
        b.load_batch([(p, m) for _, _, _, p, m in reps])
        b.prepare()
        b.step(3)
        out.append([b.export_replica(r) for r in range(len(reps))])
        b.close()
    for r in range(len(reps)):
        assert out[0][r][0].tobytes() == out[1][r][0].tobytes()
        assert out[0][r][1].tobytes() == out[1][r][1].tobytes()


def test_batch_rejects_polymerising_rules(product):
    reps = _replicas(2, seed=13)
    cfg, replicas = scenes.batch_of(reps)
    rules = scenes.test_rules()   # holds a polymerising transition
    with pytest.raises(product.ScError):
        product.Simulation(cfg, scenes.test_types(), rules, replicas=replicas)


def test_batch_rejects_a_replica_too_small_for_its_periodic_box(product):
    reps = _replicas(2, seed=14)
    cfg, replicas = scenes.batch_of(reps)
    replicas[1].sim_size = 2.0 * cfg.grid_cell_size
    with pytest.raises(product.ScError):
        product.Simulation(cfg, reps[0][1], reps[0][2], replicas=replicas)


@pytest.mark.gpu
def test_generated_batch_equals_generated_solo_sims(product):
    """sc_generate_batch gives every replica the scene sc_generate_uniform
    gives a sim of its own; two steps later they still agree bit for bit."""
    specs = scenes.batch_specs(6, seed=21, n_lo=500, n_hi=4000)
    cfg, replicas = scenes.batch_sim_args(specs)
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    kinds = (scenes.LIPID, scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B)
    batch = product.Simulation(cfg, types, rules, replicas=replicas)
    batch.generate_batch([x[0] for x in specs], [x[1] for x in specs], kinds, [x[3] for x in specs],
                         [x[4] for x in specs])
    batch.prepare()
    batch.step(2)
    for r, (n, nm, box, mix, sd) in enumerate(specs):
        c = scenes.measured_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box, seed=sd)
        solo = product.Simulation(c, types, rules)
        solo.generate_uniform(n, nm, kinds, mix, sd)
        solo.prepare()
        solo.step(2)
        assert_same_state(batch.export_replica(r), solo.export_state(), species=c.num_metabolites,
                          what=f"generated replica {r}")
        solo.close()
    batch.close()


@pytest.mark.gpu
def test_scene_batch_replicas_equal_their_own_sims(product):
    """A batch of structured scenes (sc_generate_scene_batch): each replica
    -- generated one replica at a time into its own slots, then stepped with
    the others -- equals a sim of its own with sc_generate_scene and that seed."""
    box = 120.0
    groups = scenes.vesicle_groups(box, shell_r=50.0, lipids=2000, interior=3000, complexes=20, complex_size=20)
    n = abi.scene_particles(groups)
    nm = 4000
    seeds = [5, 9, 11]
    cfg = abi.make_config(num_particles=n, num_metabolic_particles=nm, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8, seed=5,
                          periodic=0, walls=1, pair_claim=1, rule_probabilities=1, noise_coordination_steps=4,
                          relaxation_steps=6, metabolite_diffusion_steps=3)
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    replicas = [abi.Replica(n + 16 * r, nm + 8, box, 0, sd) for r, sd in enumerate(seeds)]
    batch = product.Simulation(cfg, types, rules, replicas=replicas)
    batch.generate_scene_batch(groups, nm, seeds)
    batch.prepare()
    batch.step(2)
    for r, sd in enumerate(seeds):
        c = abi.config_from_bytes(bytes(cfg))
        c.num_particles, c.num_metabolic_particles, c.seed = n + 16 * r, nm + 8, sd
        solo = product.Simulation(c, types, rules)
        solo.generate_scene(groups, nm, sd)
        solo.prepare()
        solo.step(2)
        assert_same_state(batch.export_replica(r), solo.export_state(), species=cfg.num_metabolites,
                          what=f"scene replica {r}")
        solo.close()
    batch.close()
