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

from oracle import build as obuild  # noqa: E402
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


def scene_tables():
    """The shipped tables (universe-config/gen/large-molecules.json, 179 types;
    complexification.json, 648 rules with 396 transitions and 64
    polymerisations) on a dense walled box of lipids and the partner types
    of the rules that complexify forms directly."""
    from spatial_cell_gb300 import native
    gen = os.path.join(os.path.dirname(os.path.dirname(obuild.REFERENCE_SRC)), "universe-config", "gen")
    types = native.load_types_json(os.path.join(gen, "large-molecules.json"))
    rules = native.load_rules_json(os.path.join(gen, "complexification.json"))
    direct = rules[rules["only_via_transition"] == 0]
    kinds = sorted({int(t) for t in np.concatenate([direct["first_partner_type"], direct["second_partner_type"]])
                    if t >= 0 and types["radius"][t] > 0})
    n, nm, box = 1600, 1200, 44.0
    rng = np.random.default_rng(91)
    ty = np.where(rng.random(n) < 0.2, 0, rng.choice(kinds, n)).astype(np.int32)
    p = scenes.blank_particles(n)
    p["id"] = np.arange(n, dtype=np.int32)
    p["type"] = ty
    p["radius"] = types["radius"][ty]
    p["hydrophobic"] = types["hydrophobic"][ty]
    p["pos"] = (rng.random((n, 3)) * box).astype(np.float32)
    p["rot"] = scenes.random_quaternions(rng, n)
    m = scenes.uniform_metabolic(rng, nm, box, types, 10)
    cfg = abi.make_config(num_particles=n + 256, num_metabolic_particles=nm, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=10, seed=91,
                          steps=10, relaxation_steps=6, metabolite_diffusion_steps=3, periodic=0)
    return cfg, types, rules, p, m, n


SCENES = {"golden_mixed": scene_mixed, "golden_workload": scene_workload, "golden_tables": scene_tables}


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
    for n in (sys.argv[1:] or SCENES):
        print(generate(n), os.path.getsize(os.path.join(HERE, n + ".npz")))
