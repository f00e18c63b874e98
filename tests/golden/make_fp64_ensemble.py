"""Generates tests/golden/fp64_ensemble.npz: ensemble observables of the FP64
host oracle after 1000 steps, the reference point of the FP32 device
ensemble (tests/test_gpu_fp64_ensemble.py).

    python tests/golden/make_fp64_ensemble.py [--seeds 1-16] [--steps 1000]

Each ensemble member is a periodic cube at the small workload's number
density (65,536 particles per (200 nm)^3) and physics -- its rules (A + B
bind with probability 0.1 per step), pair claim, 6 nm cells -- reduced to
4,096 particles + 8,192 metabolic items (a 79.4 nm box), its initial state
drawn with numpy from the member's seed (scenes.uniform_particles /
uniform_metabolic).  The oracle is oracle/scport.cpp built with double
precision state and arithmetic (kind "port64"); its final state, exported
to the reference's float records, gives the observables that
oracle/observables.py computes in double precision: MSD and mean |v|^2 of
particles and of metabolic items, active counts, bond slots, and the
histogram of particle pair distances below 6 nm in 12 bins.  Per-member
values are stored, so the test can state the ensemble's own spread.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import observables as obs  # noqa: E402
from oracle.engine import OracleEngine, max_threads, set_threads  # noqa: E402
from spatial_cell_gb300 import scenes  # noqa: E402

N, NM, STEPS, R_MAX, BINS = 4096, 8192, 1000, 6.0, 12
OUT = os.path.join(HERE, "fp64_ensemble.npz")


def member(seed, n=N, nm=NM):
    """(config, types, rules, particles, metabolic) of ensemble member `seed`."""
    box = float(200.0 * (n / 65536.0) ** (1.0 / 3.0))
    cfg = scenes.measured_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box, seed=seed)
    rng = np.random.default_rng(seed)
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    p = scenes.uniform_particles(rng, n, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, nm, cfg.sim_size, types, cfg.num_metabolites)
    return cfg, types, rules, p, m


def observables(pc, mc, org_p, org_m, box):
    """The member's observables from exported float records (double sums)."""
    op = obs.observe(pc, org_p, box, True, bonds=True)
    om = obs.observe(mc, org_m, box, True)
    h = obs.pair_histogram(pc, -1, -1, R_MAX, BINS, box, True)
    return dict(msd_p=op["msd"], msd_m=om["msd"], v2_p=op["mean_v2"], v2_m=om["mean_v2"], active_p=op["active"],
                active_m=om["active"], bonds=op["bond_slots"], hist=h.astype(np.float64))


def run(kind, seed, steps):
    cfg, types, rules, p, m = member(seed)
    e = OracleEngine(kind, cfg, types, rules)
    e.load_state(p, m)
    e.prepare()
    p0, m0 = e.export_state()
    org_p, org_m = obs.mark(p0), obs.mark(m0)
    e.step(steps)
    pc, mc = e.export_state()
    e.close()
    return observables(pc, mc, org_p, org_m, cfg.sim_size)


def save(path, seeds, rows, steps):
    out = {k: np.array([r[k] for r in rows]) for k in rows[0]}
    np.savez_compressed(path, seeds=np.array(seeds), steps=steps, n=N, nm=NM, r_max=R_MAX, bins=BINS, **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", default="1-16")
    ap.add_argument("--steps", type=int, default=STEPS)
    ap.add_argument("--out", default=OUT)
    ap.add_argument("--append", action="store_true", help="keep the members already in --out, add the others")
    a = ap.parse_args()
    lo, _, hi = a.seeds.partition("-")
    seeds = list(range(int(lo), int(hi or lo) + 1))
    set_threads(max_threads())
    done, rows = [], []
    if a.append and os.path.exists(a.out):
        d = np.load(a.out)
        assert int(d["steps"]) == a.steps
        done = [int(x) for x in d["seeds"]]
        rows = [{k: d[k][i] for k in d.files if k not in ("seeds", "steps", "n", "nm", "r_max", "bins")}
                for i in range(len(done))]
    for s in seeds:
        if s in done:
            continue
        t0 = time.time()
        rows.append(run("port64", s, a.steps))
        done.append(s)
        print(f"seed {s}: {time.time() - t0:.0f} s, msd_p {rows[-1]['msd_p']:.4f} msd_m {rows[-1]['msd_m']:.4f}",
              flush=True)
        save(a.out, done, rows, a.steps)  # after every member: an interrupted run keeps what it made


if __name__ == "__main__":
    main()
