"""The launch-configuration autotuner (spatial_cell_gb300/autotune.py)."""
import pytest

from spatial_cell_gb300 import autotune, scenes


def _cfg(**kw):
    return scenes.workload_config("plain_small", num_particles=4096, num_metabolic_particles=8192,
                                  sim_size=200.0 * (4096 / 65536.0) ** (1.0 / 3.0), **kw)


def test_candidates_respect_the_ranges_and_the_box():
    cfg = _cfg()
    cands = autotune.candidates(cfg, cells=(5.0, 6.0, 7.0, 8.0, 30.0))
    cells = sorted({c for c, _, _ in cands})
    assert cells == [6.0, 7.0, 8.0]  # 5 < the 6 nm diffusion range; 30 leaves < 3 cells of a 79 nm box
    assert len(cands) == 3 * 2 * 2


def test_tune_picks_the_fastest_and_breaks_ties_deterministically():
    cfg = _cfg()
    cost = {6.0: 3.0, 7.0: 1.0, 8.0: 2.0}
    best, times = autotune.tune(cfg, timer=lambda c, f, t: cost[c] + 0.5 * t)
    assert best == (7.0, 0, 0)
    assert len(times) == 12
    cfg2 = autotune.apply(cfg, best)
    assert cfg2.grid_cell_size == 7.0 and cfg2.class_streams == 1 and cfg2.tiles == 0
    assert cfg2.num_particles == cfg.num_particles and cfg2.seed == cfg.seed


def test_no_candidate_is_an_error():
    with pytest.raises(ValueError):
        autotune.tune(_cfg(), cells=(4.0,), timer=lambda *a: 1.0)


@pytest.mark.gpu
def test_tuned_config_runs_and_matches_the_oracle(product):
    """The tuner times real candidates on the device; the configuration it
    picks steps bit for bit like the oracle."""
    import numpy as np
    from oracle.engine import OracleEngine
    from tests.helpers import assert_same_state
    n, nm = 2048, 4096
    cfg = scenes.workload_config("plain_small", num_particles=n, num_metabolic_particles=nm,
                                 sim_size=200.0 * (n / 65536.0) ** (1.0 / 3.0), seed=9)
    best, times = autotune.tune(cfg, steps=2, cells=(6.0, 8.0))
    assert best in times and all(t > 0 for t in times.values())
    cfg2 = autotune.apply(cfg, best)
    rng = np.random.default_rng(9)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, cfg2.sim_size, types)
    m = scenes.uniform_metabolic(rng, nm, cfg2.sim_size, types, cfg2.num_metabolites)
    gpu = product.Simulation(cfg2, types, rules)
    cpu = OracleEngine("port", cfg2, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=n)
        e.prepare()
        e.step(2)
    assert_same_state(gpu.export_state(), cpu.export_state(), species=cfg2.num_metabolites, what="tuned config")
    gpu.close()
