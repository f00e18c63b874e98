"""The device's FP32 ensemble after 1000 steps against the FP64 oracle's.

tests/golden/fp64_ensemble.npz holds, per ensemble member, the observables
of the oracle built in double precision (oracle/scport.cpp, kind "port64")
after 1000 steps, computed from its exported state by oracle/observables.py:
MSD and mean |v|^2 of particles and of metabolic items, bond slots, and the
histogram of particle pair distances below 6 nm in 12 bins (g(r) up to its
shell volumes).  tests/golden/make_fp64_ensemble.py made it and defines the
members: the small workload's density and physics (A + B bind with
probability 0.1, pair claim, periodic, 6 nm cells) reduced to 4,096
particles + 8,192 metabolic items in a 79.4 nm box, initial states drawn
with numpy from the member's seed.

The device runs the same members in single precision, all at once as one
batched sim (each replica evolves exactly as a sim of its own), and the
same host code reduces each replica's exported state.  FP32 and FP64
trajectories separate within a few hundred steps (the dynamics is chaotic),
so the two ensembles are independent samples of one process and agree only
to their sampling error: the test checks that the trajectories did
separate, that particle MSD and the pair-distance histogram agree within
1 %, and that every ensemble mean agrees within 1 % or three standard errors
of the difference, whichever is larger (the spread of the metabolic MSD
between members, about 6 %, puts its standard error near 1 % at this
ensemble size).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fp64_ensemble.npz")
QUANTITIES = ("msd_p", "msd_m", "v2_p", "v2_m", "bonds")


def _device_ensemble(product, g, seeds):
    from spatial_cell_gb300 import scenes
    members = [g.member(s) for s in seeds]
    cfg, replicas = scenes.batch_of([(c, t, r, p, m) for c, t, r, p, m in members])
    types, rules = members[0][1], members[0][2]
    batch = product.Simulation(cfg, types, rules, replicas=replicas)
    batch.load_batch([(p, m) for _, _, _, p, m in members])
    batch.prepare()
    batch.step(g.STEPS)
    out = []
    for r, (c, _, _, p, m) in enumerate(members):
        pc, mc = batch.export_replica(r)
        org_p = {int(i): q.copy() for i, q in zip(p["id"], p["pos"])}
        org_m = {int(i): q.copy() for i, q in zip(m["id"], m["pos"])}
        out.append(g.observables(pc, mc, org_p, org_m, c.sim_size))
    batch.close()
    return out


def test_fp32_ensemble_matches_fp64_oracle(product):
    from tests.golden import make_fp64_ensemble as g
    ref = np.load(FIXTURE)
    seeds = [int(s) for s in ref["seeds"]]
    assert int(ref["steps"]) == g.STEPS and int(ref["n"]) == g.N and len(seeds) >= 16
    dev = _device_ensemble(product, g, seeds)
    # the FP32 trajectories separated from the FP64 ones
    sep = np.array([abs(x["msd_p"] - r) / r for x, r in zip(dev, ref["msd_p"])])
    assert np.median(sep) > 1e-3, "device and FP64 trajectories did not separate"
    report = {}
    for q in QUANTITIES:
        a = np.array([x[q] for x in dev], np.float64)
        b = np.asarray(ref[q], np.float64)
        rel = (a.mean() - b.mean()) / b.mean()
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b)) / b.mean()
        report[q] = (rel, se)
    ha = np.sum([x["hist"] for x in dev], axis=0)
    hb = np.asarray(ref["hist"], np.float64).sum(axis=0)
    big = hb >= 1000
    hist_rel = np.abs(ha[big] - hb[big]).sum() / hb[big].sum()
    msg = (f"{len(seeds)} members; " + "; ".join(f"{q} {r:+.4f} (s.e. {s:.4f})" for q, (r, s) in report.items())
           + f"; pair-distance histogram L1 {hist_rel:.4f}")
    print(msg)
    assert abs(report["msd_p"][0]) <= 0.01, msg
    assert hist_rel <= 0.01, msg
    for q, (rel, se) in report.items():
        assert abs(rel) <= max(0.01, 3.0 * se), msg
