"""The sm_103a step against the reference's own CUDA step on the same GPU.

oracle/_ref/ref_step.cubin is the reference's kernels
(spatial_cell_sim/src/*.cuh, unmodified) compiled for sm_103a, and
oracle/ref_device.cu replays main.cu's launch sequence around them with the
CUDA toolkit's CUB sort (the reference's own step, on the GPU).  These tests
compare the product with it bit for bit in the reference's walled box with
its complexify: phase by phase on a scene with every branch except
polymerisation (whose atomicAdd slot order is left to thread scheduling in the
reference), and over whole steps at the small workload's full size.  The
cubin is built where the reference tree is present; without it the tests
are skipped.
"""
import os

import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from tests.helpers import assert_same_counters, assert_same_state, step_phases

pytestmark = pytest.mark.gpu


def _ref_device(cfg, types, rules):
    from oracle import build
    from oracle.engine import OracleEngine
    if not os.path.exists(build.ref_cubin_path()):
        pytest.skip("no oracle/_ref/ref_step.cubin (built where the reference tree is present)")
    return OracleEngine("ref_device", cfg, types, rules)


def _no_polymerisation(rules):
    r = rules.copy()
    r["polymerize"] = -1
    return r


# Stores the reference makes outside its buffers, by design of its code:
# updateGridRanges writes gridRanges[-2] and [-1] where the active items end
# (grid.cuh:61-72).
ALLOWED_GUARD_WRITES = {("rangesP", -8), ("rangesP", -4), ("rangesM", -8), ("rangesM", -4)}


def _check_guards(ref):
    stray = [g for g in ref.guards() if g not in ALLOWED_GUARD_WRITES]
    assert not stray, f"the reference stored outside its buffers: {stray}"


@pytest.mark.parametrize("seed", [0, 1])
def test_lockstep_with_the_reference_on_the_gpu(product, seed):
    cfg, types, rules, p, m, nid = scenes.test_scene(seed, n=900, nm=1800, box=42.0)
    rules = _no_polymerisation(rules)
    ref = _ref_device(cfg, types, rules)
    gpu = product.Simulation(cfg, types, rules)
    for e in (gpu, ref):
        e.load_state(p, m, step=0, next_particle_id=nid)
    prep = [(abi.PHASE_SORT_PARTICLES, 0), (abi.PHASE_SORT_METABOLIC, 0), (abi.PHASE_REMOVE_INTERFERING, 0),
            (abi.PHASE_COMPLEXIFY, -1)]
    for k, (ph, arg) in enumerate(prep + step_phases(cfg) * 2):
        gpu.run_phase(ph, arg)
        ref.run_phase(ph, arg)
        what = f"after phase #{k} ({ph}, {arg})"
        assert_same_state(gpu.export_state(), ref.export_state(), species=cfg.num_metabolites, what=what)
        assert_same_counters(gpu.counters(), ref.counters(), what=what)
        if ph in (abi.PHASE_SORT_PARTICLES, abi.PHASE_SORT_METABOLIC):
            which = 0 if ph == abi.PHASE_SORT_PARTICLES else 1
            assert np.array_equal(gpu.export_grid(which)[0], ref.export_grid(which)[0]), what
    _check_guards(ref)
    gpu.close()
    ref.close()


def test_small_workload_whole_steps_as_the_reference(product):
    """65,536 + 131,072 items in the reference's walled 200 nm box with its
    complexify (the A + B rule): prepare and two whole steps, every state
    field, counter, cell range and the reduced frame."""
    cfg = scenes.workload_config("plain_small", periodic=0, walls=0)
    rng = np.random.default_rng(cfg.seed)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, cfg.num_particles, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, cfg.num_metabolic_particles, cfg.sim_size, types, cfg.num_metabolites)
    ref = _ref_device(cfg, types, rules)
    gpu = product.Simulation(cfg, types, rules)
    for e in (gpu, ref):
        e.load_state(p, m, step=0, next_particle_id=len(p))
        e.prepare()
    for k in (1, 2):
        gpu.step(1)
        ref.step(1)
        what = f"step {k}"
        assert_same_state(gpu.export_state(), ref.export_state(), species=cfg.num_metabolites, what=what)
        assert_same_counters(gpu.counters(), ref.counters(), what=what)
        for which in (0, 1):
            assert np.array_equal(gpu.export_grid(which)[0], ref.export_grid(which)[0]), (what, which)
    rg, rr = gpu.reduce_frame(), ref.reduce_frame()
    assert rg[0].tobytes() == rr[0].tobytes() and rg[1].tobytes() == rr[1].tobytes(), "reduced frame differs"
    assert ref.nonfinite() == (0, 0)
    gp, _ = gpu.export_state()
    assert (gp["n_active_interactions"] > 0).sum() > 0
    _check_guards(ref)
    gpu.close()
    ref.close()
