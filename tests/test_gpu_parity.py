"""Parity of the sm_103a step with the CPU oracle (bit-exact).

The oracle (oracle/scport.cpp) is itself pinned to the reference's own
kernels (tests/test_oracle_ref.py) and to committed golden vectors
(tests/test_golden.py).  Here the CUDA path is driven through the C ABI
(libspatialcell.so) and compared with the oracle on the same input state:
phase by phase in lock step, over whole steps, and on the sort results.
Floating-point fields are compared as bit patterns.
"""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state, step_phases

pytestmark = pytest.mark.gpu


def _engines(product, scene):
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m, nid = scene
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=nid)
    return cfg, gpu, cpu


def _same(cfg, gpu, cpu, what):
    assert_same_state(gpu.export_state(), cpu.export_state(), species=cfg.num_metabolites, what=what)
    assert_same_counters(gpu.counters(), cpu.counters(), what=what)


@pytest.mark.parametrize("seed,periodic,walls", [(0, 0, 0), (1, 0, 0), (2, 1, 0), (3, 1, 0), (4, 0, 1)])
def test_lockstep_every_phase(product, seed, periodic, walls):
    """Prepare + two steps, comparing the whole state after every kernel
    (reference walls, and the periodic box extension)."""
    cfg, gpu, cpu = _engines(product, scenes.test_scene(seed, n=900, nm=1800, box=42.0, periodic=periodic,
                                                        walls=walls))
    prep = [(abi.PHASE_SORT_PARTICLES, 0), (abi.PHASE_SORT_METABOLIC, 0), (abi.PHASE_REMOVE_INTERFERING, 0),
            (abi.PHASE_COMPLEXIFY, -1)]
    seq = prep + step_phases(cfg) * 2
    for k, (ph, arg) in enumerate(seq):
        gpu.run_phase(ph, arg)
        cpu.run_phase(ph, arg)
        _same(cfg, gpu, cpu, f"after phase #{k} ({ph}, {arg})")


def test_sort_permutation_and_ranges(product):
    """Stable sort permutation and the reference's gridRanges layout."""
    cfg, gpu, cpu = _engines(product, scenes.test_scene(5, n=1200, nm=2500, box=45.0))
    gpu.prepare()
    cpu.prepare()
    for step in range(2):
        for which, ph in ((0, abi.PHASE_SORT_PARTICLES), (1, abi.PHASE_SORT_METABOLIC)):
            gpu.run_phase(ph)
            cpu.run_phase(ph)
            rg, pg = gpu.export_grid(which)
            rc, pc = cpu.export_grid(which)
            assert np.array_equal(pg, pc), f"permutation differs (set {which})"
            assert np.array_equal(rg, rc), f"cell ranges differ (set {which})"
        gpu.step(1)
        cpu.step(1)


@pytest.mark.parametrize("species,periodic", [(10, 0), (8, 0), (8, 1)])
def test_whole_steps(product, species, periodic):
    cfg, gpu, cpu = _engines(product, scenes.test_scene(7, n=1500, nm=3000, box=48.0, species=species,
                                                        periodic=periodic))
    gpu.prepare()
    cpu.prepare()
    gpu.step(3)
    cpu.step(3)
    _same(cfg, gpu, cpu, "after 3 steps")
    rg = gpu.reduce_frame()
    rc = cpu.reduce_frame()
    assert rg[0].tobytes() == rc[0].tobytes(), "reduced particle frame differs"
    assert rg[1].tobytes() == rc[1].tobytes(), "reduced metabolic frame differs"


@pytest.mark.parametrize("periodic,tiles,streams,pairs", [(1, 1, 1, 0), (0, 1, 1, 0), (1, 0, 1, 0), (0, 0, 1, 0),
                                                           (1, 0, 3, 0), (0, 0, 3, 0), (1, 0, 1, 1), (0, 0, 3, 1)])
def test_measured_workload_small(product, periodic, tiles, streams, pairs):
    """The measured workload's physics at a reduced size (same density), with
    the metabolic sweeps on shared-memory tiles and on per-item lists (4-byte
    entries, or 16-byte entries with the frozen geometry), and the particle
    work classes on one stream or forked onto three."""
    cfg = scenes.workload_config("plain_small", num_particles=8192, num_metabolic_particles=16384, sim_size=100.0,
                                 seed=3, periodic=periodic, tiles=tiles, class_streams=streams, metabolic_pairs=pairs)
    rng = np.random.default_rng(3)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, cfg.num_particles, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, cfg.num_metabolic_particles, cfg.sim_size, types, cfg.num_metabolites)
    cfg_, gpu, cpu = _engines(product, (cfg, types, rules, p, m, len(p)))
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, "measured workload, 2 steps")
    gp, _ = gpu.export_state()
    assert (gp["n_active_interactions"] > 0).sum() > 0, "the A+B rule formed no bond"


def test_deterministic(product):
    scene = scenes.test_scene(9, n=1000, nm=2000, box=40.0)
    runs = []
    for _ in range(2):
        cfg, types, rules, p, m, nid = scene
        s = product.Simulation(cfg, types, rules)
        s.load_state(p, m, next_particle_id=nid)
        s.prepare()
        s.step(2)
        runs.append(s.export_state())
        s.close()
    assert runs[0][0].tobytes() == runs[1][0].tobytes()
    assert runs[0][1].tobytes() == runs[1][1].tobytes()


@pytest.mark.parametrize("limit,periodic,tiles,pairs",
                         [(0, 0, 1, 0), (2, 0, 1, 0), (2, 1, 1, 0), (2, 1, 0, 0), (3, 0, 0, 0), (5, 1, 0, 0),
                          (9, 1, 0, 0), (12, 0, 0, 0), (3, 1, 0, 1), (9, 0, 0, 1)])
def test_pair_list_overflow_paths(product, limit, periodic, tiles, pairs):
    """Items whose pair list overflows are handled by scanning their
    neighbourhood, or, once the overflow pools have grown to their demand at a
    synchronisation, by walking their whole lists there (a thread per short
    list, a warp per long one); with the list capacity capped, the paths run
    side by side and must still match the oracle bit for bit."""
    scene = scenes.test_scene(8, n=900, nm=1800, box=42.0, periodic=periodic)
    scene[0].pair_list_limit = limit
    scene[0].tiles = tiles
    scene[0].metabolic_pairs = pairs
    cfg, gpu, cpu = _engines(product, scene)
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, f"2 steps with pair lists capped at {limit}")
    gpu.sync()  # the overflow pools grow to their demand
    for e in (gpu, cpu):
        e.step(2)
    _same(cfg, gpu, cpu, f"2 more steps on the grown overflow pools, lists capped at {limit}")


@pytest.mark.parametrize("streams", [1, 3])
def test_step_graphs_equal_direct_launches(product, streams):
    """Steps replayed from captured CUDA graphs give the bytes of steps
    launched phase by phase (several steps: both buffer parities replayed),
    with the particle work classes on one stream or forked onto three."""
    scene = scenes.test_scene(12, n=900, nm=1800, box=42.0, periodic=1)
    out = []
    for graphs in (1, 0):
        cfg, types, rules, p, m, nid = scene
        cfg.class_streams = streams
        cfg.graphs = graphs
        s = product.Simulation(cfg, types, rules)
        s.load_state(p, m, next_particle_id=nid)
        s.prepare()
        s.step(5)
        out.append((s.export_state(), s.counters()))
        s.close()
    (a, ca), (b, cb) = out
    assert a[0].tobytes() == b[0].tobytes()
    assert a[1].tobytes() == b[1].tobytes()
    assert (ca.step, ca.n_active_particles, ca.kernel_launches) == (cb.step, cb.n_active_particles, cb.kernel_launches)


@pytest.mark.parametrize("drop", ["metabolic", "particles", "both"])
def test_empty_sets(product, drop):
    """A state without metabolic items, without particles, or with neither:
    the step runs and matches the oracle (capacities stay non-zero)."""
    cfg, types, rules, p, m, nid = scenes.test_scene(14, n=900, nm=1800, box=42.0, periodic=1)
    if drop in ("metabolic", "both"):
        m = m[:0]
    if drop in ("particles", "both"):
        p = p[:0]
        nid = 0
    cfg_, gpu, cpu = _engines(product, (cfg, types, rules, p, m, nid))
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, f"2 steps without {drop}")


def test_inactive_items_inside_the_range(product):
    """Items flagged inactive among active ones (the reference's gaps after
    removals) are sorted past the cells and left untouched."""
    cfg, types, rules, p, m, nid = scenes.test_scene(15, n=900, nm=1800, box=42.0)
    p = p.copy()
    m = m.copy()
    p["flags"][::7] &= ~abi.PARTICLE_FLAG_ACTIVE
    m["flags"][::5] &= ~abi.PARTICLE_FLAG_ACTIVE
    cfg_, gpu, cpu = _engines(product, (cfg, types, rules, p, m, nid))
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, "2 steps with inactive items")


def test_capacity_exactly_full(product):
    """Active counts equal to the capacities (no slack slot anywhere)."""
    cfg, types, rules, p, m, nid = scenes.test_scene(16, n=700, nm=1300, box=40.0, capacity_slack=0)
    cfg.num_metabolic_particles = len(m)
    cfg_, gpu, cpu = _engines(product, (cfg, types, rules, p, m, nid))
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, "2 steps at full capacity")


@pytest.mark.parametrize("pairs", [0, 1])
def test_metabolic_pool_grows_and_results_do_not_change(product, pairs):
    """A metabolic pair pool too small for the lists: the blocks it has no
    room for scan their neighbourhoods, the pool grows at the next
    synchronisation, and every step matches the oracle bit for bit."""
    scene = scenes.test_scene(15, n=900, nm=1800, box=42.0, periodic=1)
    scene[0].pool_per_item = 2
    scene[0].metabolic_pairs = pairs
    cfg, gpu, cpu = _engines(product, scene)
    for e in (gpu, cpu):
        e.prepare()
        e.step(1)
    _same(cfg, gpu, cpu, "1 step on a short pool")
    gpu.sync()  # grows the pool
    for ph, a in [(abi.PHASE_SORT_PARTICLES, 0), (abi.PHASE_SORT_METABOLIC, 0), (abi.PHASE_RELAX_METAB, 0)]:
        for e in (gpu, cpu):
            e.run_phase(ph, a)
    assert gpu.list_overflows()[1] == 0, "the grown pool still overflows"
    _same(cfg, gpu, cpu, "after the pool grew")
    for e in (gpu, cpu):
        e.step(2)
    _same(cfg, gpu, cpu, "2 more steps")


@pytest.mark.parametrize("kind", ["uniform", "mixed"])
def test_metabolic_fields_no_kernel_touches(product, kind):
    """The metabolic records' interaction slots, last state-change step and
    scheduled polymerisation pass through steps unchanged: one shared value
    of each (kept as two numbers), or per-record values (kept per item)."""
    cfg, types, rules, p, m, nid = scenes.test_scene(8, n=600, nm=1400, box=36.0)
    rng = np.random.default_rng(8)
    if kind == "uniform":
        m["last_state_change_step"] = 7
        m["scheduled_polymerization"] = 3
    else:
        m["last_state_change_step"] = rng.integers(-1, 50, len(m))
        m["scheduled_polymerization"] = rng.integers(-1, 4, len(m))
        k = rng.integers(0, 9, len(m))
        m["n_active_interactions"] = k
        m["interactions"] = rng.integers(0, 1000, m["interactions"].shape)
    cfg_, gpu, cpu = _engines(product, (cfg, types, rules, p, m, nid))
    for e in (gpu, cpu):
        e.prepare()
        e.step(2)
    _same(cfg, gpu, cpu, f"{kind} metabolic record fields, 2 steps")
    got = gpu.export_state()[1]
    act = (got["flags"] & 1) != 0
    ids = got["id"][act]
    for f in ("last_state_change_step", "scheduled_polymerization", "n_active_interactions"):
        assert np.array_equal(got[f][act], m[f][ids]), f


def test_load_rejects_more_than_eight_interactions_and_recovers(product):
    """sc_load_state refuses a particle with more than 8 interactions (found on
    the device as the records are unpacked, chunk by chunk) and leaves the sim
    unloaded; a correct state loads afterwards."""
    from spatial_cell_gb300.native import ScError
    cfg, types, rules, p, m, nid = scenes.test_scene(9, n=700, nm=1400, box=38.0)
    bad = p.copy()
    bad["n_active_interactions"][123] = 9
    gpu = product.Simulation(cfg, types, rules)
    with pytest.raises(ScError, match="particle 123 has more than 8 interactions"):
        gpu.load_state(bad, m, step=0, next_particle_id=nid)
    with pytest.raises(ScError):
        gpu.step(1)
    gpu.load_state(p, m, step=0, next_particle_id=nid)
    from oracle.engine import OracleEngine
    cpu = OracleEngine("port", cfg, types, rules)
    cpu.load_state(p, m, step=0, next_particle_id=nid)
    for e in (gpu, cpu):
        e.prepare()
        e.step(1)
    _same(cfg, gpu, cpu, "after a refused load")
