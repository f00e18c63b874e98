"""Parallel polymerize (k_poly_count / _offsets / _plan / _apply / _finish)
against the oracle's one-item-at-a-time polymerize in slot order
(oracle/scport.cpp, interactions.cuh:558-740): thousands of scheduled items
at once, items whose previous monomer is itself scheduled or shared (the
serial path), and a capacity that runs out part way (the reference's
lastActive still advances past it).  Bit-exact state and counters."""
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state

pytestmark = pytest.mark.gpu


def _run(product, scene, phases, steps=0):
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m, nid = scene
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=nid)
    for ph in phases:
        gpu.run_phase(ph, 0)
        cpu.run_phase(ph, 0)
    assert_same_state(gpu.export_state(), cpu.export_state(), species=cfg.num_metabolites, what="after polymerize")
    assert_same_counters(gpu.counters(), cpu.counters(), what="after polymerize")
    c = gpu.counters()
    if steps:
        gpu.step(steps)
        cpu.step(steps)
        assert_same_state(gpu.export_state(), cpu.export_state(), species=cfg.num_metabolites, what="after steps")
        assert_same_counters(gpu.counters(), cpu.counters(), what="after steps")
    gpu.close()
    cpu.close()
    return c


PHASES = (abi.PHASE_SORT_PARTICLES, abi.PHASE_SORT_METABOLIC, abi.PHASE_POLYMERIZE)


@pytest.mark.parametrize("pairs", [1, 100, 6000])
def test_many_scheduled_items_at_once(product, pairs):
    """Every controller creates a monomer in the same pass (6,000 > the old
    one-CTA list of 4,096), then two whole steps."""
    c = _run(product, scenes.polymer_scene(11, pairs), PHASES, steps=2)
    assert c.n_active_particles >= 3 * pairs


@pytest.mark.parametrize("sched,shared", [(40, 0), (0, 40), (25, 25)])
def test_conflicting_items_run_in_slot_order(product, sched, shared):
    """Previous monomers that are themselves scheduled, or shared by two
    controllers: the one-thread path in slot order."""
    _run(product, scenes.polymer_scene(12, 3000, scheduled_monomers=sched, shared=shared), PHASES, steps=1)


@pytest.mark.parametrize("slack", [0, 1, 777])
def test_capacity_runs_out(product, slack):
    """Fewer free slots than new monomers: the first `slack` in slot order
    are created, lastActive advances by all of them."""
    c = _run(product, scenes.polymer_scene(13, 2000, capacity_slack=slack), PHASES)
    assert c.n_active_particles == 4000 + slack
