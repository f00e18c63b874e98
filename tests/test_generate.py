"""The device scene generator (sc_generate_uniform, csrc/sc_gen.h).

CPU tests check the generator's records (built by the oracle from the same
definition) for the properties the scene promises; the GPU test checks that
the device writes exactly those records and that a generated sim steps like
one loaded with them."""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_state

KINDS = [scenes.LIPID, scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B]


def _gen(n=20000, nm=40000, box=80.0, species=8, seed=5, fractions=(0.4, 0.3, 0.2, 0.1)):
    from oracle.engine import generate_uniform
    return generate_uniform(n, nm, KINDS, fractions, scenes.baseline_types(), box, species, seed)


def test_generated_scene_properties():
    box, species = 80.0, 8
    p, m = _gen(box=box, species=species)
    types = scenes.baseline_types()
    assert (p["id"] == np.arange(len(p))).all() and (m["id"] == np.arange(len(m))).all()
    assert (p["flags"] == abi.PARTICLE_FLAG_ACTIVE).all() and (m["type"] == 1000).all()
    for recs in (p, m):
        assert (recs["pos"] >= 0).all() and (recs["pos"] < box).all()
        assert np.allclose(np.linalg.norm(recs["rot"], axis=1), 1.0, atol=1e-5)
        assert (recs["last_state_change_step"] == -1).all() and (recs["scheduled_polymerization"] == -1).all()
        assert (recs["angular_velocity"][:, 3] == 1.0).all() and (recs["n_active_interactions"] == 0).all()
    share = np.array([(p["type"] == k).mean() for k in KINDS])
    assert np.allclose(share, [0.4, 0.3, 0.2, 0.1], atol=0.02)
    assert (p["radius"] == types["radius"][p["type"]]).all()
    slab = m["pos"][:, 0] < box * np.float32(0.2)
    assert (m["metabolites"][slab, 0] == 100.0).all() and (m["metabolites"][~slab, 0] == 0.0).all()
    assert (m["metabolites"][:, 1:species] >= 0).all() and (m["metabolites"][:, 1:species] < 10).all()
    assert (m["metabolites"][:, species:] == 0).all()


def test_generator_is_a_function_of_seed_and_index():
    a, am = _gen(n=1000, nm=500, seed=9)
    b, bm = _gen(n=3000, nm=800, seed=9)
    assert a.tobytes() == b[:1000].tobytes() and am.tobytes() == bm[:500].tobytes()
    c, _ = _gen(n=1000, nm=500, seed=10)
    assert a.tobytes() != c.tobytes()


@pytest.mark.gpu
def test_device_generation_equals_oracle_and_steps_alike(product):
    n, nm, box, seed = 6000, 12000, 73.0, 21
    cfg = scenes.workload_config("plain_small", num_particles=n + 64, num_metabolic_particles=nm + 64, sim_size=box,
                                 seed=7)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    fr = (0.4, 0.4, 0.1, 0.1)
    p, m = _gen(n=n, nm=nm, box=box, species=cfg.num_metabolites, seed=seed, fractions=fr)
    g = product.Simulation(cfg, types, rules)
    g.generate_uniform(n, nm, KINDS, fr, seed)
    ref = product.Simulation(cfg, types, rules)
    ref.load_state(p, m)
    assert_same_state(g.export_state(), ref.export_state(), species=cfg.num_metabolites, what="generated state")
    for s in (g, ref):
        s.prepare()
        s.step(2)
    assert_same_state(g.export_state(), ref.export_state(), species=cfg.num_metabolites, what="2 steps")
    g.close()
    ref.close()
