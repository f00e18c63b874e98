"""propagateState (sc_config.propagate_state; interactions.cuh:743-822,
whose launch the reference's step leaves commented out) on the GPU against
the oracle's pass, which tests/test_oracle_ref.py pins to the reference
kernel: as one phase, and inside whole steps (graph-captured) with the switch
on.  Bit-exact state and counters."""
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state

pytestmark = pytest.mark.gpu


def _pair(product, scene):
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


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_propagate_phase(product, seed):
    scene = scenes.propagation_scene(seed)
    cfg, gpu, cpu = _pair(product, scene)
    for ph in (abi.PHASE_SORT_PARTICLES, abi.PHASE_SORT_METABOLIC, abi.PHASE_PROPAGATE_STATE):
        gpu.run_phase(ph, 0)
        cpu.run_phase(ph, 0)
    _same(cfg, gpu, cpu, "after propagateState")
    changed = (gpu.export_state()[0]["state"][: len(scene[3])] != scene[3]["state"]).sum()
    assert changed > 50


@pytest.mark.parametrize("periodic", [0, 1])
def test_steps_with_propagation(product, periodic):
    cfg, types, rules, p, m, nid = scenes.propagation_scene(7)
    cfg.periodic = periodic
    cfg, gpu, cpu = _pair(product, (cfg, types, rules, p, m, nid))
    gpu.prepare()
    cpu.prepare()
    for k in range(3):
        gpu.step(1)
        cpu.step(1)
        _same(cfg, gpu, cpu, f"after step {k + 1}")
