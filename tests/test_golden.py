"""Golden vectors of the reference's own kernels (tests/golden/*.npz,
generated by tests/golden/make_golden.py from the reference harness).

The CPU oracle must reproduce them byte for byte (so the oracle stays pinned
to the reference where the reference tree is absent); the sm_103a step must
reproduce every state field, counter, sort result and frames.dat record."""
import os

import numpy as np
import pytest

from spatial_cell_gb300 import abi
from tests.helpers import assert_same_state, diff_fields

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["golden_mixed", "golden_workload", "golden_tables"]


def _load(name):
    g = dict(np.load(os.path.join(HERE, name + ".npz")))
    cfg = abi.config_from_bytes(g["config"].tobytes())
    # rule records are 96 bytes in every layout version; view them in the current one
    g["rules"] = np.frombuffer(g["rules"].tobytes(), abi.RULE_DTYPE)
    return g, cfg


def _run(engine, g):
    engine.load_state(g["p_in"], g["m_in"], step=0, next_particle_id=int(g["next_particle_id"]))
    out = {}
    engine.prepare()
    out["prepared"] = engine.export_state()
    for k in (1, 2):
        engine.step(1)
        out[f"step{k}"] = engine.export_state()
        c = engine.counters()
        out[f"counters_step{k}"] = np.array([c.n_active_particles, c.n_active_metabolic_particles,
                                             c.next_particle_id, c.step], np.int32)
    out["frame"] = engine.reduce_frame()
    for which, ph in ((0, abi.PHASE_SORT_PARTICLES), (1, abi.PHASE_SORT_METABOLIC)):
        engine.run_phase(ph)
        out[f"grid{which}"] = engine.export_grid(which)
    return out


def _check(out, g, species, exact_bytes):
    for tag, key in (("prepared", "prepared"), ("step1", "step1"), ("step2", "step2")):
        got_p, got_m = out[key]
        want_p, want_m = g[f"p_{tag}"], g[f"m_{tag}"]
        if exact_bytes:
            problems = diff_fields(got_p, want_p) + diff_fields(got_m, want_m)
            assert not problems, f"{tag}: " + "\n".join(problems)
        else:
            assert_same_state((got_p, got_m), (want_p, want_m), species=species, what=tag)
    for k in (1, 2):
        assert np.array_equal(out[f"counters_step{k}"], g[f"counters_step{k}"])
    assert out["frame"][0].tobytes() == g["frame_p"].tobytes()
    assert out["frame"][1].tobytes() == g["frame_m"].tobytes()
    for which in (0, 1):
        r, perm = out[f"grid{which}"]
        assert np.array_equal(perm, g[f"perm_{which}"])
        assert np.array_equal(r, g[f"ranges_{which}"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    from oracle.engine import OracleEngine
    g, cfg = _load(name)
    e = OracleEngine("port", cfg, g["types"], g["rules"])
    _check(_run(e, g), g, cfg.num_metabolites, exact_bytes=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(product, name):
    g, cfg = _load(name)
    s = product.Simulation(cfg, g["types"], g["rules"])
    _check(_run(s, g), g, cfg.num_metabolites, exact_bytes=False)
    s.close()
