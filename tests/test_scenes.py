"""Structured device scenes (sc_generate_scene, csrc/sc_gen.h): shells,
balls, lattice complexes and wrapped chains.

CPU tests check the records the oracle builds from the shared definition
for the geometry and bonds each group kind promises; the GPU test checks
that the device writes exactly those records and that the generated walled
vesicle steps bit for bit like the oracle."""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state


def _types():
    t = scenes.test_types()
    return t


def _gen(groups, nm=0, box=120.0, species=8, seed=5, types=None):
    from oracle.engine import generate_scene
    return generate_scene(groups, nm, _types() if types is None else types, box, species, seed)


def _small_vesicle(box=120.0):
    return scenes.vesicle_groups(box, shell_r=50.0, lipids=2000, interior=3000, complexes=20, complex_size=20)


def test_group_layout_ids_and_counts():
    groups = _small_vesicle()
    p, _ = _gen(groups)
    n = abi.scene_particles(groups)
    assert len(p) == n == 2000 + 3000 + 20 * 20
    assert (p["id"] == np.arange(n)).all()
    assert (p["flags"] == abi.PARTICLE_FLAG_ACTIVE).all()
    assert (p["pos"] >= 0).all() and (p["pos"] <= 120.0).all()
    assert np.allclose(np.linalg.norm(p["rot"], axis=1), 1.0, atol=1e-5)


def test_shell_leaflets_radius_and_orientation():
    box = 120.0
    c = np.full(3, box / 2, np.float32)
    groups = _small_vesicle(box)
    p, _ = _gen(groups)
    n_out = int(groups[0]["count"][0])
    outer, inner = p[:n_out], p[n_out:2000]
    for recs, r, sign in ((outer, 50.0, 1.0), (inner, 46.0, -1.0)):
        d = recs["pos"] - c
        dist = np.linalg.norm(d, axis=1)
        assert np.allclose(dist, r, rtol=1e-5)
        assert (recs["type"] == scenes.LIPID).all()
        # up = rot applied to (0, 1, 0): radial outward on the outer leaflet, inward on the inner one
        q = recs["rot"].astype(np.float64)
        x, y, z, w = q.T
        up = np.stack([2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x)], axis=1)
        cosang = (up * d).sum(1) / dist
        assert (sign * cosang > 0.999).all()
    # uniform on the sphere: each octant holds about an eighth
    oct_ = ((outer["pos"] - c) > 0).astype(int) @ np.array([1, 2, 4])
    share = np.bincount(oct_, minlength=8) / len(outer)
    assert np.allclose(share, 1 / 8, atol=0.03)


def test_interior_ball_and_mix():
    box = 120.0
    groups = _small_vesicle(box)
    p, _ = _gen(groups)
    ball = p[2000:5000]
    assert (np.linalg.norm(ball["pos"] - box / 2, axis=1) <= 40.0 + 1e-4).all()
    share = np.array([(ball["type"] == k).mean() for k in (scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B)])
    assert np.allclose(share, [0.70, 0.15, 0.15], atol=0.03)
    assert (ball["n_active_interactions"] == 0).all()


def test_complexes_are_lattice_trees():
    groups = _small_vesicle()
    p, _ = _gen(groups)
    cx = p[5000:].reshape(20, 20)
    for comp in cx:
        pos = comp["pos"].astype(np.float64)
        # sites sit on a cubic lattice of spacing 3 in the complex's frame: pairwise distances are
        # 3 * sqrt(integer), and no two sites coincide
        d2 = ((pos[:, None] - pos[None]) ** 2).sum(-1) / 9.0
        iu = np.triu_indices(20, 1)
        assert np.allclose(d2[iu], np.round(d2[iu]), atol=1e-3) and (np.round(d2[iu]) >= 1).all()
        assert (comp["rot"] == comp["rot"][0]).all()
        ids = set(comp["id"].tolist())
        edges = 0
        for r in comp:
            for btype, bgroup, bpartner in r["interactions"][: r["n_active_interactions"]]:  # (type, group, partner)
                assert btype == abi.INTERACTION_TYPE_CHAIN and bpartner in ids
                partner = comp[comp["id"] == bpartner][0]
                back = {(int(x[2]), int(x[1])) for x in partner["interactions"][: partner["n_active_interactions"]]}
                other = abi.INTERACTION_GROUP_BACKWARD if bgroup == abi.INTERACTION_GROUP_FORWARD \
                    else abi.INTERACTION_GROUP_FORWARD
                assert (int(r["id"]), other) in back
                # bonded sites are lattice neighbours
                assert abs(np.linalg.norm(r["pos"] - partner["pos"]) - 3.0) < 1e-3
                edges += bgroup == abi.INTERACTION_GROUP_FORWARD
        assert edges == 19  # a spanning tree of the 20 sites


def test_wrapped_chains_follow_the_reference_step():
    t = _types()
    kinds = [scenes.CHAIN_A, scenes.CHAIN_B, scenes.CHAIN_C]
    g = abi.scene_group(abi.SCENE_WRAPPED_CHAINS, 5, kinds, center=(100.0, 100.0, 100.0), radius=20.0, unit=12,
                        link_type=abi.INTERACTION_TYPE_CHAIN)
    p, _ = _gen([g], box=200.0)
    ch = p.reshape(5, 12)
    for chain in ch:
        assert (chain["type"] == np.array([kinds[k % 3] for k in range(12)])).all()
        for k in range(1, 12):
            # step length radius(type - 1) + radius(type), along the member's up vector
            step = np.linalg.norm(chain["pos"][k] - chain["pos"][k - 1])
            ty = chain["type"][k]
            assert abs(step - (t["radius"][ty - 1] + t["radius"][ty])) < 1e-4
            assert chain["interactions"][k][0][2] == chain["id"][k - 1]  # slot 0: (type, group, partner)
            assert chain["interactions"][k][0][1] == abi.INTERACTION_GROUP_BACKWARD
        assert chain["n_active_interactions"][0] == 1 and chain["n_active_interactions"][-1] == 1
        assert (chain["n_active_interactions"][1:-1] == 2).all()


def test_fibonacci_shell_matches_the_reference_spiral():
    n = 1600
    g = abi.scene_group(abi.SCENE_FIBONACCI_SHELL, n, [scenes.LIPID], center=(60.0, 60.0, 60.0), radius=0.0)
    p, _ = _gen([g])
    # the reference's count-based radius and its spiral, in double precision
    r = np.sqrt(n / 1000.0 * (1.0 / 2.5) ** 2) * 40.0
    gr = (np.sqrt(5.0) + 1.0) / 2.0
    ga = (2.0 - gr) * (2.0 * np.pi)
    i = np.arange(1, n + 1)
    lat = np.arcsin(-1.0 + 2.0 * i / (n + 1))
    lon = ga * i
    pts = np.stack([np.cos(lon) * np.cos(lat), np.sin(lon) * np.cos(lat), np.sin(lat)], axis=1)
    assert np.allclose(p["pos"], 60.0 + pts * r, atol=2e-4)


def test_scene_is_a_function_of_seed_group_and_unit():
    a, _ = _gen(_small_vesicle(), seed=3)
    b, _ = _gen(_small_vesicle(), seed=3)
    c, _ = _gen(_small_vesicle(), seed=4)
    assert a.tobytes() == b.tobytes() and a.tobytes() != c.tobytes()
    # a group's records do not depend on the groups after it
    d, _ = _gen(_small_vesicle()[:2], seed=3)
    assert d.tobytes() == a[:2000].tobytes()


@pytest.mark.parametrize("bad", [
    dict(kind=9), dict(count=-1), dict(kind=abi.SCENE_COMPLEXES, unit=65, spacing=3.0),
    dict(kind=abi.SCENE_COMPLEXES, unit=4, spacing=0.0), dict(kind=abi.SCENE_WRAPPED_CHAINS, unit=3, kinds=[0]),
])
def test_invalid_groups_are_refused(bad):
    kw = dict(kind=abi.SCENE_UNIFORM_BALL, count=10, kinds=[scenes.DUMMY], radius=5.0)
    kw.update(bad)
    g = abi.scene_group(kw.pop("kind"), kw.pop("count"), kw.pop("kinds"), **kw)
    with pytest.raises(ValueError):
        _gen([g])


@pytest.mark.gpu
def test_device_vesicle_equals_oracle_and_steps_bit_exact(product):
    from oracle.engine import OracleEngine
    box = 120.0
    groups = _small_vesicle(box)
    n, nm, seed = abi.scene_particles(groups), 9000, 17
    cfg = abi.make_config(num_particles=n + 64, num_metabolic_particles=nm + 64, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8, seed=5,
                          steps=10, periodic=0, walls=1)
    types, rules = _types(), scenes.baseline_rules()
    p, m = _gen(groups, nm=nm, box=box, species=cfg.num_metabolites, seed=seed, types=types)
    g = product.Simulation(cfg, types, rules)
    g.generate_scene(groups, nm, seed)
    cpu = OracleEngine("port", cfg, types, rules)
    cpu.load_state(p, m, step=0, next_particle_id=n)
    assert_same_state(g.export_state(), cpu.export_state(), species=cfg.num_metabolites, what="generated vesicle")
    for s in (g, cpu):
        s.prepare()
        s.step(2)
    assert_same_state(g.export_state(), cpu.export_state(), species=cfg.num_metabolites, what="vesicle, 2 steps")
    assert_same_counters(g.counters(), cpu.counters(), what="vesicle, 2 steps")
    g.close()
