"""Complexify extensions on the CPU oracle: a per-rule binding probability and
the deterministic pair claim (sc_config.pair_claim).

The reference's complexify (interactions.cuh:216-346) appends a bond on the
scanning particle's side only, so two particles can both bond a third that
keeps only one of them (its TODO at interactions.cuh:297).  The pair claim
forms rule bonds only between particles that hold each other's claim key,
so every rule bond is recorded on both sides.  Rules with a probability bind
with that probability per step, from one Philox draw per (rule, step, pair)
that both partners see alike.
"""
import json

import numpy as np

from spatial_cell_gb300 import abi, scenes


def dense_ab_scene(seed=1, n=3000, box=60.0, probability=None, claim=0, walls=0):
    """Only A and B particles at high density: many particles have several
    partners in reach at once."""
    rng = np.random.default_rng(seed)
    types = scenes.baseline_types()
    rules = scenes.baseline_rules(probability=probability)
    p = scenes.uniform_particles(rng, n, box, types, fractions=((scenes.TYPE_A, 0.5), (scenes.DUMMY, 0.0),
                                                              (scenes.TYPE_B, 0.5)))
    m = scenes.uniform_metabolic(rng, 64, box, types, 8)
    cfg = abi.make_config(num_particles=n, num_metabolic_particles=64, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8,
                          seed=100 + seed, noise_coordination_steps=2, relaxation_steps=2,
                          metabolite_diffusion_steps=1, pair_claim=claim, walls=walls,
                          rule_probabilities=int(probability is not None))
    return cfg, types, rules, p, m


def rule_bonds(p):
    """{(id, partner id, rule id)} of the active particles' rule bonds (type >= 10)."""
    out = set()
    for rec in p[(p["flags"] & abi.PARTICLE_FLAG_ACTIVE) != 0]:
        for k in range(int(rec["n_active_interactions"])):
            t, g, pid = (int(x) for x in rec["interactions"][k])
            if t >= 10:
                out.add((int(rec["id"]), pid, t))
    return out


def unreciprocated(p):
    b = rule_bonds(p)
    return {(a, c, t) for a, c, t in b if (c, a, t) not in b}


def _run(scene, steps=2):
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m = scene
    e = OracleEngine("port", cfg, types, rules)
    e.load_state(p, m)
    e.prepare()
    out = [e.export_state()[0]]
    for _ in range(steps):
        e.step(1)
        out.append(e.export_state()[0])
    e.close()
    return out


def test_reference_complexify_leaves_one_sided_bonds():
    """The reference's scan at this density: some particle records a bond its
    partner does not (the over-subscription its TODO names)."""
    states = _run(dense_ab_scene(claim=0), steps=1)
    assert rule_bonds(states[0]), "no bond formed"
    assert unreciprocated(states[0]), "expected one-sided bonds from the reference's scan"


def test_pair_claim_bonds_are_always_mutual():
    states = _run(dense_ab_scene(claim=1), steps=2)
    for s in states:
        assert not unreciprocated(s)
    assert len(rule_bonds(states[-1])) > len(rule_bonds(states[0])) > 0
    # the A + B rule has a group: at most one such bond per particle
    for s in states:
        act = s[(s["flags"] & 1) != 0]
        assert (act["n_active_interactions"] <= 1).all()


def test_pair_claim_is_deterministic_and_keyed_by_distance():
    a = _run(dense_ab_scene(seed=3, claim=1), steps=1)
    b = _run(dense_ab_scene(seed=3, claim=1), steps=1)
    assert a[-1].tobytes() == b[-1].tobytes()
    # the first claims: each bonded pair is the closest open pair of both partners
    cfg, types, rules, p, m = dense_ab_scene(seed=3, claim=1)
    pos = {int(r["id"]): r["pos"].astype(np.float64) for r in p}
    for pid, qid, _ in rule_bonds(a[0]):
        assert np.all(np.abs(pos[qid] - pos[pid]) <= 5.5 + 1e-6)


def test_probability_zero_one_and_between():
    never = _run(dense_ab_scene(seed=2, probability=0.0), steps=2)
    assert not any(rule_bonds(s) for s in never)
    always = _run(dense_ab_scene(seed=2, probability=1.0), steps=2)
    plain = _run(dense_ab_scene(seed=2, probability=None), steps=2)
    for x, y in zip(always, plain):
        assert x.tobytes() == y.tobytes()
    some = _run(dense_ab_scene(seed=2, probability=0.1), steps=1)
    n_some, n_all = len(rule_bonds(some[0])), len(rule_bonds(plain[0]))
    assert 0 < n_some < 0.8 * n_all  # a particle tries several partners per step, each at 0.1


def test_probability_draw_is_the_same_from_both_sides():
    """With the claim and a probability both partners see one draw: bonds stay mutual."""
    states = _run(dense_ab_scene(seed=4, probability=0.3, claim=1), steps=3)
    assert rule_bonds(states[-1])
    for s in states:
        assert not unreciprocated(s)


def test_probability_bytes_are_ignored_unless_enabled():
    """Reference rule records leave their padding unset: garbage there must not
    change anything unless the sim asks for rule probabilities."""
    cfg, types, rules, p, m = dense_ab_scene(seed=5)
    junk = rules.copy()
    junk["use_probability"] = 121
    junk["probability"] = 1e-30
    a = _run((cfg, types, rules, p, m), steps=1)
    b = _run((cfg, types, junk, p, m), steps=1)
    assert a[-1].tobytes() == b[-1].tobytes()


def test_rule_loader_reads_probability(product, tmp_path):
    path = tmp_path / "rules.json"
    path.write_text(json.dumps([
        {"id": 5, "group": 5, "firstPartnerType": 2, "secondPartnerType": 3, "relativeOrientation": [0, 0, 0, 1],
         "relativePosition": [0, 5, 0], "probability": 0.1},
        {"id": 6, "group": 6, "firstPartnerType": 2, "secondPartnerType": 2, "relativeOrientation": [0, 0, 0, 1],
         "relativePosition": [0, 5, 0]},
    ]))
    r = product.load_rules_json(str(path))
    assert list(r["use_probability"]) == [1, 0]
    assert r["probability"][0] == np.float32(0.1) and r["probability"][1] == 0.0


def test_config_loader_reads_the_extension_keys(product, tmp_path):
    path = tmp_path / "config.json"
    path.write_text(json.dumps({"simSize": 100.0, "pairClaim": 1, "ruleProbabilities": 1}))
    c = product.load_config_json(str(path))
    assert c.pair_claim == 1 and c.rule_probabilities == 1 and c.sim_size == 100.0
