"""Pins the CPU oracle (oracle/scport.cpp) to the reference itself.

oracle/_ref/libscref.so is the reference's own kernel code
(spatial_cell_sim/src/*.cuh) compiled for the host from the reference tree
(oracle/build.py, oracle/ref_harness.cpp).  Both run the same scenario and
must agree byte for byte: every phase in lock step, whole steps, the sort
permutation and cell ranges, and frames.dat records.  The setup-surface
loaders of the product (config.json, large-molecules.json,
complexification.json) are pinned to the reference's jsoncpp loaders.

These tests need the reference tree, which only exists where the oracle is
developed; elsewhere they are skipped and tests/test_golden.py carries the
pin (golden vectors generated by the reference harness).
"""
import os

import numpy as np
import pytest

from oracle import build as obuild
from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state, diff_fields, step_phases

pytestmark = pytest.mark.skipif(not obuild.reference_available(), reason="reference tree not present")

REF_ROOT = os.path.dirname(os.path.dirname(obuild.REFERENCE_SRC))


def _pair(scene):
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m, nid = scene
    a = OracleEngine("port", cfg, types, rules)
    b = OracleEngine("ref", cfg, types, rules)
    for e in (a, b):
        e.load_state(p, m, step=0, next_particle_id=nid)
    return cfg, a, b


def _bytes_equal(a, b, what):
    pa, ma = a.export_state()
    pb, mb = b.export_state()
    problems = diff_fields(pa, pb) + diff_fields(ma, mb)
    assert not problems, f"{what}:\n" + "\n".join(problems)
    assert_same_counters(a.counters(), b.counters(), what)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_whole_steps_byte_identical(seed):
    cfg, port, ref = _pair(scenes.test_scene(seed, n=1200, nm=2400, box=44.0))
    port.prepare()
    ref.prepare()
    _bytes_equal(port, ref, "after prepare")
    for k in range(3):
        port.step(1)
        ref.step(1)
        _bytes_equal(port, ref, f"after step {k + 1}")
    rp, rq = port.reduce_frame(), ref.reduce_frame()
    assert rp[0].tobytes() == rq[0].tobytes() and rp[1].tobytes() == rq[1].tobytes()


def test_every_phase_in_lockstep():
    cfg, port, ref = _pair(scenes.test_scene(4, n=800, nm=1600, box=40.0))
    prep = [(abi.PHASE_SORT_PARTICLES, 0), (abi.PHASE_SORT_METABOLIC, 0), (abi.PHASE_REMOVE_INTERFERING, 0),
            (abi.PHASE_COMPLEXIFY, -1)]
    for k, (ph, arg) in enumerate(prep + step_phases(cfg) * 2):
        port.run_phase(ph, arg)
        ref.run_phase(ph, arg)
        _bytes_equal(port, ref, f"phase #{k} ({ph}, {arg})")


def test_sort_results():
    cfg, port, ref = _pair(scenes.test_scene(6, n=1500, nm=3000, box=46.0))
    port.prepare()
    ref.prepare()
    port.step(1)
    ref.step(1)
    for which, ph in ((0, abi.PHASE_SORT_PARTICLES), (1, abi.PHASE_SORT_METABOLIC)):
        port.run_phase(ph)
        ref.run_phase(ph)
        r1, p1 = port.export_grid(which)
        r2, p2 = ref.export_grid(which)
        assert np.array_equal(p1, p2)
        assert np.array_equal(r1, r2)


def test_measured_workload_physics():
    """The A+B rule workload (same densities, reduced size) over 3 steps."""
    cfg = scenes.workload_config("plain_small", num_particles=6000, num_metabolic_particles=12000, sim_size=90.0,
                                 num_metabolites=10, seed=5, periodic=0)
    rng = np.random.default_rng(5)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, cfg.num_particles, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, cfg.num_metabolic_particles, cfg.sim_size, types, 10)
    cfg, port, ref = _pair((cfg, types, rules, p, m, len(p)))
    for e in (port, ref):
        e.prepare()
        e.step(3)
    _bytes_equal(port, ref, "3 steps")


def test_scene_exercises_every_branch():
    """The differential scenes reach transitions, state changes, breaks and
    polymerisation (so the byte-identity above covers those paths)."""
    cfg, port, _ = _pair(scenes.test_scene(0, n=1200, nm=2400, box=44.0))
    p0, m0 = port.export_state()
    port.prepare()
    port.step(3)
    p1, m1 = port.export_state()
    c = port.counters()
    n0 = 1200
    assert c.n_active_particles > n0, "no monomer was polymerised"
    live = p1[: c.n_active_particles]
    assert (live["last_state_change_step"] >= 0).any(), "no transition set a state"
    types_ = live["interactions"][:, :, 0][np.arange(8)[None] < live["n_active_interactions"][:, None]]
    assert (types_ == abi.INTERACTION_TYPE_CHAIN).any() and (types_ >= 1001).any() and (types_ == 0).any()
    assert (m1["flags"][: c.n_active_metabolic_particles] & 1).sum() < c.n_active_metabolic_particles, \
        "no metabolic particle was removed for overlapping a lipid"


def test_table_loaders_match_reference(product):
    """sc_types_load_json / sc_rules_load_json + sc_create's flattening versus
    loadParticleTypeInfo / loadComplexificationInfo / flatten* / partnerMap*
    (chemistry.cuh:10-51, interactions.cuh:17-145) on the shipped tables."""
    import ctypes
    from oracle.engine import load
    gen = os.path.join(REF_ROOT, "universe-config", "gen")
    types = product.load_types_json(os.path.join(gen, "large-molecules.json"))
    rules = product.load_rules_json(os.path.join(gen, "complexification.json"))
    _, f = load("ref")
    cap = 4096
    rt = np.zeros(cap, abi.TYPE_INFO_DTYPE)
    rf = np.zeros(cap, abi.RULE_DTYPE)
    ri = np.zeros(cap * 2, np.int32)
    rp = np.zeros(cap, abi.RULE_DTYPE)
    n = [ctypes.c_int(0) for _ in range(4)]
    sim_dir = os.path.join(REF_ROOT, "spatial_cell_sim")
    rc = f["load_tables"](sim_dir.encode(), abi.ptr(rt), cap, ctypes.byref(n[0]), abi.ptr(rf), cap,
                          ctypes.byref(n[1]), abi.ptr(ri), cap * 2, ctypes.byref(n[2]), abi.ptr(rp), cap,
                          ctypes.byref(n[3]))
    assert rc == 0
    assert len(types) == n[0].value
    assert types.tobytes() == rt[: n[0].value].tobytes()
    flat = np.zeros(n[1].value, abi.RULE_DTYPE)
    for r in rules:
        if (flat[r["id"]]["id"] == 0) and r["id"] >= 0:
            flat[r["id"]] = r
    # field by field, the reference's fields only: it leaves its padding (where the extension fields sit) unset
    assert not diff_fields(flat[abi.RULE_REFERENCE_FIELDS], rf[: n[1].value][abi.RULE_REFERENCE_FIELDS])
    assert not flat["use_probability"].any()   # no shipped rule has a "probability" key
    # one rule with an explicit "polymerize": null reads as 0, as jsoncpp's asInt() of null
    nulls = [r for r in rules if r["id"] in (1730, 1740)]
    assert nulls and all(r["polymerize"] == 0 for r in nulls)
    # partner index: same [start, end) sizes per type and the same rule multiset
    # (the reference's order within a type is std::unordered_map iteration order)
    idx = ri[: n[2].value].reshape(-1, 2)
    pr = rp[: n[3].value]
    by_type = {}
    for r in rules:
        for t in (r["first_partner_type"], r["second_partner_type"]):
            if t >= 0:
                by_type.setdefault(int(t), []).append(int(r["id"]))
    for t, ids in by_type.items():
        s, e = idx[t]
        assert sorted(ids) == sorted(int(x) for x in pr[s:e]["id"])


def test_config_loader_matches_reference(product, tmp_path):
    import ctypes
    from oracle.engine import load
    _, f = load("ref")
    path = os.path.join(REF_ROOT, "spatial_cell_sim", "config.json")
    mine = product.load_config_json(path)
    theirs = abi.make_config()
    ng, nb = ctypes.c_int(0), ctypes.c_int(0)
    assert f["load_config"](path.encode(), ctypes.byref(theirs), ctypes.byref(ng), ctypes.byref(nb)) == 0
    for k, _ in abi.Config._fields_:
        if k in ("num_metabolites", "seed", "periodic") or k.startswith("_"):
            continue
        assert getattr(mine, k) == getattr(theirs, k), k
    assert product.grid(mine) == (ng.value, nb.value)
    # grid derivation on other sizes (config.cuh:65-74)
    for size, cell in [(200.0, 6.0), (635.0, 6.0), (900.0, 6.0), (10.0, 10.0), (1.0, 10.0), (47.9, 6.0)]:
        p = tmp_path / "c.json"
        p.write_text(f'{{"simSize": {size}, "gridCellSize": {cell}}}')
        c1 = product.load_config_json(str(p))
        c2 = abi.make_config()
        assert f["load_config"](str(p).encode(), ctypes.byref(c2), ctypes.byref(ng), ctypes.byref(nb)) == 0
        assert product.grid(c1) == (ng.value, nb.value), (size, cell)


@pytest.mark.parametrize("case", ["no_metabolic", "no_particles", "inactive_gaps", "tiny"])
def test_edge_states_byte_identical(case):
    """The port against the reference's own kernels on the states the GPU
    edge-case tests use: without metabolic items, without particles, with
    inactive items among active ones (the reference's gaps after removals),
    and a scene of a few items."""
    scene = list(scenes.test_scene(14, n=900, nm=1800, box=42.0))
    p, m = scene[3].copy(), scene[4].copy()
    if case == "no_metabolic":
        m = m[:0]
    elif case == "no_particles":
        p = p[:0]
        scene[5] = 0
    elif case == "inactive_gaps":
        p["flags"][::7] &= ~abi.PARTICLE_FLAG_ACTIVE
        m["flags"][::5] &= ~abi.PARTICLE_FLAG_ACTIVE
    else:
        p, m = p[:9], m[:17]
    scene[3], scene[4] = p, m
    cfg, port, ref = _pair(tuple(scene))
    port.prepare()
    ref.prepare()
    _bytes_equal(port, ref, f"{case}: after prepare")
    for k in range(2):
        port.step(1)
        ref.step(1)
        _bytes_equal(port, ref, f"{case}: after step {k + 1}")


@pytest.mark.parametrize("seed", [0, 1])
def test_propagate_state_byte_identical(seed):
    """propagateState (interactions.cuh:743-822), which the reference's step
    leaves commented out: the port's pass equals the reference kernel's, as
    one phase after a sort and inside whole steps with the switch on."""
    cfg, port, ref = _pair(scenes.propagation_scene(seed))
    for ph in (abi.PHASE_SORT_PARTICLES, abi.PHASE_SORT_METABOLIC, abi.PHASE_PROPAGATE_STATE):
        port.run_phase(ph, 0)
        ref.run_phase(ph, 0)
        _bytes_equal(port, ref, f"after phase {ph}")
    before = scenes.propagation_scene(seed)[3]
    after = port.export_state()[0]
    assert (after["state"][: len(before)] != before["state"]).sum() > 50, "the pass changed too few states"
    for k in range(2):
        for ph, arg in step_phases(cfg):
            port.run_phase(ph, arg)
            ref.run_phase(ph, arg)
        _bytes_equal(port, ref, f"after step {k + 1}")
