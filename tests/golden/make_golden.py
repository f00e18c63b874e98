"""Generates the golden vectors of tests/golden/ from the reference itself.

    python tests/golden/make_golden.py

Runs the reference's own kernels compiled for the host (oracle/_ref, built
from the reference tree by oracle/build.py) on small seeded scenes and saves
inputs and outputs as compressed .npz files: the state after sc_prepare's
sequence (main.cu:284-338) and after each of two steps (main.cu:347-661),
the counters, the frames.dat records, and the last sort's permutation and
cell ranges.  Only this script needs the reference tree; the tests that read
the vectors run anywhere.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.engine import OracleEngine  # noqa: E402
from spatial_cell_gb300 import abi, scenes  # noqa: E402


def scene_mixed():
    return scenes.test_scene(31, n=400, nm=800, box=34.0)


def scene_workload():
    n, nm = 1000, 2000
    box = float(635.0 * (n / 2097152) ** (1.0 / 3.0))
    cfg = scenes.workload_config("plain_large", num_particles=n, num_metabolic_particles=nm, sim_size=box,
                                 num_metabolites=10, seed=77, periodic=0)
    rng = np.random.default_rng(77)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, box, types)
    m = scenes.uniform_metabolic(rng, nm, box, types, 10)
    return cfg, types, rules, p, m, n


SCENES = {"golden_mixed": scene_mixed, "golden_workload": scene_workload}


def generate(name):
    cfg, types, rules, p, m, nid = SCENES[name]()
    e = OracleEngine("ref", cfg, types, rules)
    e.load_state(p, m, step=0, next_particle_id=nid)
    out = {"config": np.frombuffer(bytes(cfg), np.uint8), "types": types, "rules": rules, "p_in": p, "m_in": m,
           "next_particle_id": np.int32(nid)}
    e.prepare()
    out["p_prepared"], out["m_prepared"] = e.export_state()
    for k in (1, 2):
        e.step(1)
        out[f"p_step{k}"], out[f"m_step{k}"] = e.export_state()
        c = e.counters()
        out[f"counters_step{k}"] = np.array([c.n_active_particles, c.n_active_metabolic_particles,
                                             c.next_particle_id, c.step], np.int32)
    out["frame_p"], out["frame_m"] = e.reduce_frame()
    for which, ph in ((0, abi.PHASE_SORT_PARTICLES), (1, abi.PHASE_SORT_METABOLIC)):
        e.run_phase(ph)
        out[f"ranges_{which}"], out[f"perm_{which}"] = e.export_grid(which)
    e.close()
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    for n in SCENES:
        print(generate(n), os.path.getsize(os.path.join(HERE, n + ".npz")))
