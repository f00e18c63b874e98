"""Parity at the sizes the bench measures, and of the complexify extensions.

The measured workloads (bench.py) run the A + B rule at probability 0.1 per
step with complexify by pair claim, in a periodic box, with the production
settings (step graphs, particle work classes on three streams when the
particles fill the device, the metabolic pair pool sized by demand).  Here
the sm_103a step is compared with the CPU oracle bit for bit at those full
sizes: the small workload (65,536 particles + 131,072 metabolic items in a
200 nm box) over two whole steps, and the large one (2,097,152 + 8,388,608
in 635 nm) over one step; state, counters, sort permutations, cell ranges
and the reduced frame.
"""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, diff_fields, mask_state
from tests.test_complexify_ext import dense_ab_scene, unreciprocated

pytestmark = pytest.mark.gpu


def assert_same_state_chunked(sa, sb, species, what, chunk=1 << 20):
    """assert_same_state over slices of `chunk` items (large states)."""
    no_p, no_m = np.zeros(0, abi.PARTICLE_DTYPE), np.zeros(0, abi.METABOLIC_DTYPE)
    problems = []
    for k, name in enumerate(("particles", "metabolic")):
        a, b = sa[k], sb[k]
        assert a.shape == b.shape
        for s in range(0, len(a), chunk):
            pair = [(a[s:s + chunk], no_m), (b[s:s + chunk], no_m)] if k == 0 else \
                [(no_p, a[s:s + chunk]), (no_p, b[s:s + chunk])]
            x, y = (mask_state(*pair[0], species=species)[k], mask_state(*pair[1], species=species)[k])
            problems += [f"{name} [{s}, {s + len(x)}) {d}" for d in diff_fields(x, y)]
            if len(problems) > 8:
                break
    assert not problems, f"{what}: state differs\n" + "\n".join(problems)


def _engines(product, cfg, types, rules, p, m):
    from oracle.engine import OracleEngine
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=len(p))
    return gpu, cpu


def _compare_step(cfg, gpu, cpu, what):
    assert_same_state_chunked(gpu.export_state(), cpu.export_state(), cfg.num_metabolites, what)
    assert_same_counters(gpu.counters(), cpu.counters(), what=what)
    for which in (0, 1):
        rg, pg = gpu.export_grid(which)
        rc, pc = cpu.export_grid(which)
        assert np.array_equal(pg, pc), f"{what}: sort permutation differs (set {which})"
        assert np.array_equal(rg, rc), f"{what}: cell ranges differ (set {which})"


@pytest.mark.parametrize("streams", [0, 3])
def test_small_workload_at_full_size(product, streams):
    """65,536 + 131,072 items, 200 nm periodic, seed 1, p = 0.1 with pair
    claim: two whole steps, every field, counter and sort result, and the
    frame (class_streams 0 is the production choice at this size: one stream)."""
    cfg, types, rules, p, m = scenes.build_workload("plain_small", class_streams=streams)
    assert (cfg.num_particles, cfg.num_metabolic_particles, cfg.sim_size) == (65536, 131072, 200.0)
    gpu, cpu = _engines(product, cfg, types, rules, p, m)
    gpu.prepare()
    cpu.prepare()
    for k in (1, 2):
        gpu.step(1)
        cpu.step(1)
        _compare_step(cfg, gpu, cpu, f"small workload, step {k}")
    rg, rc = gpu.reduce_frame(), cpu.reduce_frame()
    assert rg[0].tobytes() == rc[0].tobytes() and rg[1].tobytes() == rc[1].tobytes(), "reduced frame differs"
    gp, _ = gpu.export_state()
    assert (gp["n_active_interactions"] > 0).sum() > 0, "no A + B bond formed"
    assert not unreciprocated(gp)
    assert np.isfinite(gp["pos"]).all()
    gpu.close()
    cpu.close()


def test_large_workload_one_step(product):
    """The bench's headline state (2,097,152 + 8,388,608 items, 635 nm
    periodic, seed 2): one whole step with the production settings, every
    field, counter and sort result."""
    cfg, types, rules, p, m = scenes.build_workload("plain_large")
    gpu, cpu = _engines(product, cfg, types, rules, p, m)
    del p, m
    gpu.prepare()
    cpu.prepare()
    gpu.step(1)
    cpu.step(1)
    _compare_step(cfg, gpu, cpu, "large workload, step 1")
    gpu.close()
    cpu.close()


@pytest.mark.parametrize("claim,probability", [(0, 0.3), (1, None), (1, 0.3)])
def test_complexify_extensions_match_the_oracle(product, claim, probability):
    cfg, types, rules, p, m = dense_ab_scene(seed=6, probability=probability, claim=claim)
    gpu, cpu = _engines(product, cfg, types, rules, p, m)
    gpu.prepare()
    cpu.prepare()
    for k in (1, 2):
        gpu.step(1)
        cpu.step(1)
        _compare_step(cfg, gpu, cpu, f"claim {claim} p {probability}, step {k}")
    if claim:
        assert not unreciprocated(gpu.export_state()[0])


@pytest.mark.parametrize("periodic", [0, 1])
def test_pair_claim_on_the_rule_scene(product, periodic):
    """The scene with every rule kind (groups, states, transitions,
    polymerisation, a homotypic rule without group) under the pair claim."""
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m, nid = scenes.test_scene(21, n=1200, nm=2000, box=44.0, periodic=periodic)
    cfg.pair_claim = 1
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=nid)
        e.prepare()
        e.step(3)
    _compare_step(cfg, gpu, cpu, "rule scene, 3 steps")
