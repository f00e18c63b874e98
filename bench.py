"""Throughput of the spatial_cell_sim step on one GB300 (particle-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload plain_large|plain_small]

A step is one iteration of the reference's step loop (main.cu:347-661) with
16 noise-coordination, 32 relaxation and 8 diffusion sub-iterations; the
metric counts particles plus metabolic particles per step.  The default
workload is the single large instance: 2,097,152 particles (lipid / dummy /
A / B = 40 / 40 / 10 / 10 %) and 8,388,608 metabolic particles of 8 species
in a 635 nm box, 6 nm cells, seeded synthetic state (no dataset exists).

``--impl ours`` prints one JSON line:
  value     device-resident step throughput (CUDA events on the sim's stream,
            state already in HBM; inputs of several GB, larger than L2);
  e2e       the same through the C ABI with host buffers: sc_load_state from
            pinned host memory, then per step sc_step + sc_reduce_frame into
            pinned host memory (the frames.dat payload, persisted every step
            as the reference does);
  roofline  the dominant kernel's algorithmic bytes per launch over its
            measured launch time, against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (oracle/scport.cpp, OpenMP on all host cores)
            timed on a same-density sub-box of the workload, and on one core;
  reference_cuda  the reference's own CUDA step (its kernels compiled for
            sm_103a, main.cu's launch sequence, CUB's sort of whole structs)
            timed on the same GPU and state beside this build's step;
  batched / serving / vesicle  the batched replica cells, the request loop
            and the crowded vesicle case (docstrings of their samples).
``--impl reference`` times the CPU implementation alone (the reference has no
CPU path of its own; its CUDA step is the reference_cuda entry above).
``--cpu-small-full`` runs the small workload in full (200 steps) on the CPU
oracle.  Under torchrun, every rank runs an independent replica (the path
does not shard); value is the sum over ranks of items per step over the
slowest rank.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from spatial_cell_gb300 import abi, scenes  # noqa: E402

METRIC = "particle-steps/s on 1 GB300, batched vs plain at tol; serving p50/p99 latency"
UNIT = "particle-steps/s"


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_seed(workload, rank):
    """Each rank steps its own replica: the workload's seed offset by the rank."""
    return scenes.WORKLOADS[workload]["seed"] + rank


def aggregate_replicas(items_per_step, steps, seconds, device=None):
    """Whole-job throughput of independent replicas: the items all ranks
    stepped over the slowest rank's time.  Returns (rate, slowest seconds).
    Without an initialised process group it is the local rate."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return items_per_step * steps / seconds, seconds
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    n = torch.tensor([float(items_per_step) * steps], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) / float(t.item()), float(t.item())


def _measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is producing (nvidia-smi takes a moment to
            # start); what it saw before the region is dropped
            t0 = time.perf_counter()
            while not self.samples and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
            self.samples.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# Algorithmic HBM bytes per launch of the step's kernels: each field a kernel
# needs read once and each field it produces written once, neighbour data
# served on chip (per-item figures of the measurement plan).
def algorithmic_bytes(phase, N, Nm, S, bbar=0.0):
    return {
        "relax": N * (104 + 12 * bbar),
        "relax_metab": Nm * 44 + N * 32,
        "relax_partners": N * 44 + Nm * 32,
        "diffuse": Nm * (16 + 8 * S),
        "coordinate_noise": N * (84 + 12 * bbar),
    }.get(phase)


def step_algorithmic_bytes(cfg, bbar):
    """Compulsory HBM bytes of one whole step: every item's fields read and
    written once per phase that depends on them, neighbour data served on
    chip, elementwise phases fused into the adjacent sweeps (per-item
    figures: particles 6,292 B and metabolic items 2,258 B at the large
    workload with no bonds)."""
    import math
    N, Nm, S = cfg.num_particles, cfg.num_metabolic_particles, cfg.num_metabolites
    C, R, D = cfg.noise_coordination_steps, cfg.relaxation_steps, cfg.metabolite_diffusion_steps
    _, bits, cells = abi.grid_dims(cfg)
    d = math.ceil((3 * bits + 1) / 8)
    P = 80 + 12 * bbar
    M = 68 + 4 * S
    per_p = (20 + 4 + 16 * d + 2 * P + 4 + 4 + 8 * cells / max(N, 1) + C * (84 + 12 * bbar) + 56
             + R * (104 + 12 * bbar) + (R / 2) * 32 + (R / 2) * 44 + 100 + 24 * bbar)
    per_m = (20 + 4 + 16 * d + 2 * M + 4 + 4 + 8 * cells / max(Nm, 1) + 120 + (R / 2) * 44 + (R / 2) * 32
             + D * (16 + 8 * S))
    return N * per_p + Nm * per_m


def measured_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` at `workload` from the committed ncu
    summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t[workload][kernel]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


PHASES = {
    "relax": abi.PHASE_RELAX,
    "relax_metab": abi.PHASE_RELAX_METAB,
    "relax_partners": abi.PHASE_RELAX_PARTNERS,
    "diffuse": abi.PHASE_DIFFUSE,
    "coordinate_noise": abi.PHASE_COORDINATE_NOISE,
    "complexify": abi.PHASE_COMPLEXIFY,
    "transition": abi.PHASE_TRANSITION,
    "apply_velocities": abi.PHASE_APPLY_VELOCITIES,
}


def per_phase_times(sim, stream, torch, reps=3):
    """Average device time of one launch of each neighbour phase (CUDA events
    on the sim's stream).  Phases that double-buffer are run in pairs so the
    state's buffer parity is unchanged afterwards.  Pair lists are built
    before the timed launches: inside a step one build serves every
    sub-iteration of a phase, and the builds are timed with the step."""
    out = {}
    # as inside a step: both sets sorted, positions in the cells they were sorted into
    sim.run_phase(abi.PHASE_SORT_PARTICLES, 0)
    sim.run_phase(abi.PHASE_SORT_METABOLIC, 0)
    for name, ph in PHASES.items():
        if name in ("complexify", "transition", "apply_velocities"):
            continue  # change the state; timed as part of the step only
        sim.run_phase(ph, 0)  # an untimed pair first builds the phase's pair list
        sim.run_phase(ph, 0)
        sim.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2 * reps):
            sim.run_phase(ph, 0)
        e1.record(stream)
        e1.synchronize()
        out[name] = e0.elapsed_time(e1) / (2 * reps)
        if name == "relax_metab":
            out["_pairs_metabolic"] = sim.pair_counts()[1]  # the list the timed launches walked
    return out


def sub_box(workload, frac):
    """Overrides giving a frac-volume box of the workload at its densities."""
    if frac == 1.0:
        return {}
    cfg0 = scenes.workload_config(workload)
    return dict(num_particles=max(1024, int(cfg0.num_particles * frac)),
                num_metabolic_particles=max(1024, int(cfg0.num_metabolic_particles * frac)),
                sim_size=float(cfg0.sim_size * frac ** (1.0 / 3.0)))


def host_threads():
    """Every host thread this process may run on (a launcher's OMP_NUM_THREADS=1
    does not apply: rank 0 runs the CPU leg alone)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_sample(args, reps=1, warmup=0, threads=None, frac=None, workload=None):
    """Times the CPU oracle on a same-density sub-box of the workload:
    `warmup` untimed steps, then `reps` timed steps, on `threads` host threads
    (default: all)."""
    from oracle import engine as oengine
    oengine.set_threads(threads or host_threads())
    frac = args.cpu_fraction if frac is None else frac
    workload = workload or args.workload
    cfg = scenes.measured_config(workload, **sub_box(workload, frac))
    n, nm, box = cfg.num_particles, cfg.num_metabolic_particles, cfg.sim_size
    rng = np.random.default_rng(cfg.seed)
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    p = scenes.uniform_particles(rng, n, box, types)
    m = scenes.uniform_metabolic(rng, nm, box, types, cfg.num_metabolites)
    e = oengine.OracleEngine("port", cfg, types, rules)
    e.load_state(p, m)
    e.prepare()
    threads = oengine.max_threads()
    if warmup:
        e.step(warmup)
    t0 = time.perf_counter()
    e.step(reps)
    dt = time.perf_counter() - t0
    e.close()
    rate = (n + nm) * reps / dt
    sample = (f"{reps} step(s) (after {warmup} untimed) of a {frac:.4g}-volume sub-box of {workload} at its "
              f"density ({n} + {nm} items, {box:.1f} nm), {dt:.1f} s")
    return rate, threads, sample


def cpu_single_core(args):
    """The CPU oracle on one host thread: 2 steps of a 1/64-volume sub-box."""
    rate, _, sample = cpu_sample(args, reps=2, threads=1, frac=1.0 / 64)
    return {"value": rate, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}


def cpu_small_full(args):
    """The small workload (65,536 + 131,072 items, 200 nm periodic, seed 1) run
    in full on the CPU oracle: all 200 of its steps on every host thread."""
    cfg = scenes.measured_config("plain_small")
    rate, threads, sample = cpu_sample(args, reps=cfg.steps, threads=host_threads(), frac=1.0, workload="plain_small")
    return {"metric": METRIC, "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "workload": "plain_small", "sample": sample}


def batched_sample(args, native, torch):
    """The batched workload: args.batch_replicas replica cells (particles
    log-uniform in [2048, 262144] from seed 3, metabolic x2, each periodic
    cube at the small workload's density, mix ~ Dirichlet(2,2,1,1)) stepped
    as ONE batched sim -- every phase one launch over all replicas, the
    replica in the high part of the sort key, each step a captured graph --
    against a sample of the same replicas stepped one at a time as sims of
    their own.  Scenes are generated on the device.  The grid cell size is
    the autotuner's pick on a sub-batch.  Device-resident timing with CUDA
    events on the sim's stream."""
    from spatial_cell_gb300 import autotune
    specs = scenes.batch_specs(args.batch_replicas)
    kinds = (scenes.LIPID, scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B)
    types, rules = scenes.baseline_types(), scenes.workload_rules()

    def make_batch(sp, cell):
        cfg, reps = scenes.batch_sim_args(sp, grid_cell_size=cell)
        b = native.Simulation(cfg, types, rules, replicas=reps)
        b.generate_batch([x[0] for x in sp], [x[1] for x in sp], kinds, [x[3] for x in sp], [x[4] for x in sp])
        b.prepare()
        return b

    def timed_steps(sim, k):
        stream = torch.cuda.ExternalStream(sim.stream_handle())
        sim.step(1)  # captures the step graph
        sim.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(k)
        e1.record(stream)
        e1.synchronize()
        sim.sync()
        return e0.elapsed_time(e1) / 1e3

    # the autotuner's cell size, timed on every 16th replica as one batch
    sub = specs[::16] or specs
    sub_items = sum(n + nm for n, nm, *_ in sub)
    times = {}
    for cell in autotune.batch_cells(scenes.measured_config("plain_small")):
        b = make_batch(sub, cell)
        times[cell] = timed_steps(b, 2) / 2
        b.close()
    cell = min(times, key=lambda c: (times[c], c))
    items = sum(n + nm for n, nm, *_ in specs)
    b = make_batch(specs, cell)
    batched_s = timed_steps(b, args.batch_steps)
    finite = all(np.isfinite(b.export_replica(r)[0]["pos"]).all() for r in (0, len(specs) // 2, len(specs) - 1))
    b.close()
    batched = items * args.batch_steps / batched_s
    # one at a time: a sample of the replicas (every 8th), each a sim of its own
    alone_items, alone_s = 0, 0.0
    k = max(2, args.batch_steps // 10)
    for n, nm, box, mix, sd in specs[::8]:
        c = scenes.measured_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box, seed=sd,
                                   grid_cell_size=cell)
        s1 = native.Simulation(c, types, rules)
        s1.generate_uniform(n, nm, kinds, mix, sd)
        s1.prepare()
        alone_s += timed_steps(s1, k)
        alone_items += (n + nm) * k
        s1.close()
    alone = alone_items / alone_s
    # one large cell of the replicas' mean composition (mix (2, 2, 1, 1) / 6, metabolic x2) at their
    # density: the single-instance rate the batch's per-item rate compares with
    n1 = 2_097_152
    c1 = scenes.measured_config("plain_small", num_particles=n1, num_metabolic_particles=2 * n1,
                                sim_size=float(200.0 * (n1 / 65536.0) ** (1.0 / 3.0)), seed=3, grid_cell_size=cell)
    s1 = native.Simulation(c1, types, rules)
    s1.generate_uniform(n1, 2 * n1, kinds, (2 / 6, 2 / 6, 1 / 6, 1 / 6), 3)
    s1.prepare()
    single_mix = 3 * n1 * args.batch_steps / timed_steps(s1, args.batch_steps)
    s1.close()
    return {"replicas": len(specs), "particles": sum(x[0] for x in specs),
            "metabolic_particles": sum(x[1] for x in specs), "steps": args.batch_steps, "value": batched,
            "unit": UNIT, "ms_per_step": 1e3 * batched_s / args.batch_steps, "state_finite": finite,
            "one_at_a_time": alone, "one_at_a_time_sample": f"{len(specs[::8])} replicas (every 8th), {k} steps each",
            "speedup": batched / alone,
            "single_instance_same_mix": {"value": single_mix, "unit": UNIT,
                                         "cell": f"{n1} particles + {2 * n1} metabolic, mix (2,2,1,1)/6, the "
                                                 "replicas' density, one sim"},
            "vs_single_instance_same_mix": batched / single_mix,
            "form": "one batched sim: one launch per phase over all replicas, replica in the high key bits, "
                    "graph-captured step",
            "sizes": "particles log-uniform in [2048, 262144] (seed 3), metabolic x2, cubes at 65,536 per "
                     "(200 nm)^3, mix Dirichlet(2,2,1,1), periodic, pair claim, A + B at p = 0.1",
            "autotuned": {"cell_nm": cell, "tuned_on": f"{len(sub)} replicas ({sub_items} items) as one batch",
                          "candidates_ms_per_step": {f"cell {c:g}": round(v * 1e3, 3) for c, v in sorted(times.items())}},
            "timing": "CUDA events on the batch's stream, after a warm-up step"}


def serving_sample(args):
    """The request loop (spatial_cell_gb300/serving.py) on a scaled-down
    stream of the serving workload: particles log-uniform in [4096, 1048576],
    metabolic x2, horizons uniform in [100, serve_horizon] steps, mix ~
    Dirichlet(1,1,1,1), the small workload's density and physics, a 160 GB
    budget.  Three runs: (1) saturated -- serve_saturated requests arriving
    at once, enough that the budget binds -- giving the server's capacity;
    (2) serve_requests requests arriving as a Poisson stream at 80 % of that
    capacity, each streaming a frame to the host every 25 steps, giving
    p50 / p99 latency and throughput; (3) the same stream served one request
    at a time.  Wall clock."""
    from spatial_cell_gb300 import serving
    hi = args.serve_horizon
    sat = serving.saturated(serving.poisson_requests(args.serve_saturated, 1.0, seed=5, h_lo=100, h_hi=hi))
    server = serving.Server(budget_bytes=160 << 30)
    t0 = time.perf_counter()
    res = server.run(sat)
    sat_s = time.perf_counter() - t0
    work = sum((r.n + r.nm) * r.horizon for r in sat)
    capacity = work / sat_s
    # the first half of the same requests through a server with room for one request at a time
    half = sat[:len(sat) // 2]
    t0 = time.perf_counter()
    serving.Server(budget_bytes=max(r.bytes for r in half)).run(half)
    sat_one = sum((r.n + r.nm) * r.horizon for r in half) / (time.perf_counter() - t0)
    peak_bytes = sum(r.bytes for r in sat)
    probe = serving.poisson_requests(args.serve_requests, 1.0, h_lo=100, h_hi=hi)
    mean_work = sum((r.n + r.nm) * r.horizon for r in probe) / len(probe)
    rate = 0.8 * capacity / mean_work
    reqs = serving.poisson_requests(args.serve_requests, rate, h_lo=100, h_hi=hi)
    live = serving.Server(budget_bytes=160 << 30, frame_every=25)
    res = live.run(reqs)
    p50, p99 = serving.percentiles(res)
    # room for one request at a time
    one = serving.Server(budget_bytes=max(r.bytes for r in reqs), frame_every=25).run(reqs)
    q50, q99 = serving.percentiles(one)
    return {"requests": len(reqs), "arrival_rate_per_s": rate, "p50_latency_s": p50, "p99_latency_s": p99,
            "value": serving.throughput(res, reqs), "unit": UNIT,
            "frames_streamed": live.frames, "frame_bytes_streamed": live.frame_bytes,
            "one_at_a_time": {"value": serving.throughput(one, reqs), "p50_latency_s": q50, "p99_latency_s": q99},
            "saturated": {"requests": len(sat), "value": capacity, "unit": UNIT, "seconds": sat_s,
                          "requests_bytes_total": peak_bytes, "budget_bytes": 160 << 30,
                          "one_at_a_time": sat_one, "one_at_a_time_sample": f"the first {len(sat) // 2} requests",
                          "speedup": capacity / sat_one},
            "stream": f"particles log-uniform [4096, 1048576], horizon uniform [100, {hi}] steps, metabolic x2, "
                      f"mix Dirichlet(1,1,1,1), 160 GB budget; latency run Poisson at 80% of the saturated "
                      f"capacity with a frame streamed every 25 steps (scaled down from 10,000 requests of "
                      f"horizons up to 5,000 steps)",
            "timing": "wall clock"}


def vesicle_sample(args, native, torch):
    """The crowded vesicle case (900 nm box with reflecting walls: 2 M lipids on a 400 nm
    bilayer shell, 6 M interior particles, 50 k 20-particle lattice complexes,
    32 M metabolic items, the measured workloads' A + B binding; counts scaled
    by --vesicle-scale), generated on the device.  One instance: particle-steps/s
    over --vesicle-steps steps after a warm-up step, with the step time at the
    start and the end and the items whose lists overflowed (they take the
    neighbourhood-scan paths).  Four replicas (seeds 5..8) on the device at
    once, each with the 4-byte metabolic pair entries (the 16-byte pool of a
    gas this dense would not leave room for four), stepped in turn for
    --vesicle-replica-steps steps.  Wall clock with the device synchronised on
    both sides."""
    cfg, groups, nm = scenes.vesicle_workload(args.vesicle_scale)
    items = cfg.num_particles + nm
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    torch.cuda.synchronize()

    def make(c, seed):
        s = native.Simulation(c, types, rules)
        s.generate_scene(groups, nm, seed)
        s.prepare()
        s.step(1)  # warm-up: captures the step graphs
        s.sync()
        return s

    one = make(cfg, cfg.seed)
    k = args.vesicle_steps
    times = []
    for _ in range(k):
        t0 = time.perf_counter()
        one.step(1)
        one.sync()
        times.append(time.perf_counter() - t0)
    ep, em = one.export_state()
    finite = bool(np.isfinite(ep["pos"][(ep["flags"] & 1) != 0]).all()
                  and np.isfinite(em["pos"][(em["flags"] & 1) != 0]).all())
    out = {"scale": args.vesicle_scale, "particles": cfg.num_particles, "metabolic_particles": nm,
           "box_nm": cfg.sim_size, "walls": "reflecting", "steps": k, "value": items * k / sum(times), "unit": UNIT,
           "ms_per_step_first_last": [round(1e3 * times[0], 1), round(1e3 * times[-1], 1)],
           "list_overflows_at_end": dict(zip(("particle", "metabolic", "lipid_metabolic", "diffusion"),
                                             one.list_overflows())),
           "device_bytes": one.device_bytes(), "state_finite": finite,
           "complexify": "pair claim, A + B bind at probability %g per step" % scenes.WORKLOAD_BIND_PROBABILITY,
           "scene": "2 leaflets r=400/396 nm (lipids uniform on each sphere), dummy/A/B 70/15/15 in the ball "
                    "r<390 nm, 20-site lattice complexes (3 nm, tree of chain bonds) in r<384 nm, metabolic "
                    "uniform in the box; generated on the device (sc_generate_scene), seed 5",
           "timing": "wall clock per step, device synchronised"}
    one.close()
    ks = args.vesicle_replica_steps
    if ks > 0:
        lean = scenes.vesicle_workload(args.vesicle_scale, metabolic_pairs=0)[0]
        seeds = [cfg.seed + r for r in range(4)]
        reps = [abi.Replica(cfg.num_particles, nm, cfg.sim_size, 0, sd) for sd in seeds]
        try:
            b = native.Simulation(lean, types, rules, replicas=reps)
        except native.ScError as e:  # the device has no room for four
            out["replicas4"] = {"not_run": f"a batch of 4 replicas could not be created: {e}"}
        else:
            b.generate_scene_batch(groups, nm, seeds)
            b.prepare()
            b.step(1)  # warm-up: captures the step graph
            b.sync()
            t0 = time.perf_counter()
            b.step(ks)
            b.sync()
            dt = time.perf_counter() - t0
            ok = all(np.isfinite(b.export_replica(r)[0]["pos"]).all() for r in range(4))
            out["replicas4"] = {"value": 4 * items * ks / dt, "unit": UNIT, "steps": ks,
                                "ms_per_step": 1e3 * dt / ks, "device_bytes": b.device_bytes(), "state_finite": ok,
                                "form": "one batched sim of 4 replicas (seeds 5..8): one launch per phase over "
                                        "all of them, graph-captured step",
                                "metabolic_pairs": "4-byte entries"}
            b.close()
    return out


def same_state_bits(a, b, species):
    """Whether two exported states hold the same bits in every field that
    carries state: interaction slots at and beyond n_active_interactions and
    metabolite species at and beyond the simulated count are left out (the
    reference keeps stale values there that no kernel reads)."""
    for x, y in zip(a, b):
        x, y = x.copy(), y.copy()
        for arr in (x, y):
            nb = np.clip(arr["n_active_interactions"], 0, abi.MAX_ACTIVE_INTERACTIONS)
            arr["interactions"][np.arange(abi.MAX_ACTIVE_INTERACTIONS)[None, :] >= nb[:, None]] = 0
            if "metabolites" in arr.dtype.names:
                arr["metabolites"][:, species:] = 0
        if x.tobytes() != y.tobytes():
            return False
    return True


def reference_cuda_sample(args, native, torch):
    """The reference's own CUDA step on this GPU beside this build's step on
    the same state: oracle/_ref/ref_step.cubin (the reference's kernels,
    compiled for sm_103a) in main.cu's launch sequence with the CUDA
    toolkit's CUB sort (oracle/ref_device.cu).  Both run the reference's
    semantics -- its walled box and its complexify, without the binding
    probability it has no notion of -- on the workload's sizes and seed.  At
    this density the reference's walled box turns positions non-finite after
    a few steps, after which its cell 0 collects every such item; steps are
    timed only while both states stay finite (checked after every step).
    Wall clock per step with the device synchronised (the reference
    synchronises inside its step); the first step of each is reported apart
    (this build captures its step graph there)."""
    from oracle import build as obuild
    from oracle.engine import OracleEngine
    if not os.path.exists(obuild.ref_cubin_path()):
        return {"unavailable": "oracle/_ref/ref_step.cubin absent (built where the reference tree is present)"}
    cfg = scenes.workload_config(args.workload, periodic=0, walls=0, **sub_box(args.workload, args.fraction))
    rng = np.random.default_rng(cfg.seed)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, cfg.num_particles, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, cfg.num_metabolic_particles, cfg.sim_size, types, cfg.num_metabolites)
    items = cfg.num_particles + cfg.num_metabolic_particles

    def finite_state(e):
        ep, em = e.export_state()
        return bool(np.isfinite(ep["pos"][(ep["flags"] & 1) != 0]).all()
                    and np.isfinite(em["pos"][(em["flags"] & 1) != 0]).all())

    def run(e, sync, finite, limit):
        times = []
        for _ in range(limit):
            t0 = time.perf_counter()
            e.step(1)
            sync()
            times.append(time.perf_counter() - t0)
            if not finite():
                return times, False
        return times, True

    ref = OracleEngine("ref_device", cfg, types, rules)
    ref.load_state(p, m)
    ref.prepare()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        ref_t, ref_ok = run(ref, lambda: None, lambda: ref.nonfinite() == (0, 0), args.ref_steps)
    ref_state = ref.export_state()
    guards = ref.guards()
    ref.close()
    sim = native.Simulation(cfg, types, rules)
    sim.load_state(p, m)
    sim.prepare()
    ours_t, ours_ok = run(sim, sim.sync, lambda: finite_state(sim), len(ref_t))
    ours_state = sim.export_state()
    sim.close()
    same = (same_state_bits(ours_state, ref_state, cfg.num_metabolites) if len(ours_t) == len(ref_t) else None)
    steady = slice(1, None) if len(ref_t) > 1 else slice(0, None)
    ref_ms = 1e3 * statistics.mean(ref_t[steady])
    ours_ms = 1e3 * statistics.mean(ours_t[steady])
    return {"kernels": "the reference's spatial_cell_sim/src/*.cuh compiled for sm_103a, launched in main.cu's "
                       "sequence with cub::DeviceRadixSort::SortPairs of whole structs",
            "config": {"particles": cfg.num_particles, "metabolic_particles": cfg.num_metabolic_particles,
                       "box_nm": cfg.sim_size, "box": "walled (clamp), the reference's", "complexify": "reference",
                       "seed": cfg.seed},
            "steps_timed": len(ref_t), "state_finite_after": ref_ok,
            "reference_ms_per_step": ref_ms, "reference_first_step_ms": 1e3 * ref_t[0],
            "reference_value": items / (ref_ms / 1e3),
            "ours_ms_per_step": ours_ms, "ours_first_step_ms": 1e3 * ours_t[0], "ours_value": items / (ours_ms / 1e3),
            "speedup": ref_ms / ours_ms, "unit": UNIT, "same_state_bits": same,
            "reference_stores_outside_buffers": guards, "clocks": clocks.summary(),
            "timing": "wall clock per step, device synchronised; mean over steps 2.. when more than one"}


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    rate, threads, sample = cpu_sample(args, reps=max(1, args.steps), warmup=max(0, args.warmup))
    cfg = scenes.workload_config(args.workload)
    line = {"metric": METRIC, "impl": "reference", "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; no dataset in the reference)",
            "config": {"workload": args.workload, "particles": cfg.num_particles,
                       "metabolic_particles": cfg.num_metabolic_particles, "box_nm": cfg.sim_size,
                       "cell_nm": cfg.grid_cell_size, "species": cfg.num_metabolites},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    from spatial_cell_gb300 import build, native

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build.build()
    cfg, types, rules, p, m = scenes.build_workload(args.workload, seed=replica_seed(args.workload, rank),
                                                    metabolic_pairs=args.metabolic_pairs,
                                                    **sub_box(args.workload, args.fraction))
    N, Nm, S = cfg.num_particles, cfg.num_metabolic_particles, cfg.num_metabolites
    items = N + Nm
    # pinned host buffers for the end-to-end leg
    p_host = torch.empty(p.nbytes, dtype=torch.uint8, pin_memory=True)
    m_host = torch.empty(m.nbytes, dtype=torch.uint8, pin_memory=True)
    p_host.numpy()[:] = p.view(np.uint8)
    m_host.numpy()[:] = m.view(np.uint8)
    # two pinned frame slots: frame k lands in slot k % 2 while step k + 1 runs
    rp_host = [torch.empty(N * abi.REDUCED_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    rm_host = [torch.empty(Nm * abi.REDUCED_METABOLIC_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
               for _ in range(2)]

    sim = native.Simulation(cfg, types, rules)
    stream = torch.cuda.ExternalStream(sim.stream_handle())
    sim.load_state(p, m)
    sim.prepare()
    for _ in range(args.warmup):
        sim.step(1)
    sim.sync()
    footprint = sim.device_bytes()

    # device-resident timing
    launches0 = sim.counters().kernel_launches
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    sim.sync()
    launches = sim.counters().kernel_launches - launches0
    value, slowest_s = aggregate_replicas(items, args.steps, ms / 1e3, device="cuda")
    ms = slowest_s * 1e3
    ms_per_step = ms / args.steps

    # per-phase breakdown (for the roofline of the dominant kernel)
    phase_ms = per_phase_times(sim, stream, torch)
    pairs = list(sim.pair_counts())  # lists as the per-phase timing left them
    pairs[1] = phase_ms.pop("_pairs_metabolic")
    counts = {"relax": cfg.relaxation_steps, "relax_metab": (cfg.relaxation_steps + 1) // 2,
              "relax_partners": (cfg.relaxation_steps + 1) // 2, "diffuse": cfg.metabolite_diffusion_steps,
              "coordinate_noise": cfg.noise_coordination_steps}
    share = {k: phase_ms[k] * counts[k] / ms_per_step for k in phase_ms}
    # the dominant single kernel: the relax phase is three class kernels run
    # concurrently, each below relax_metab's share (launch list in profiles/)
    dom = max((k for k in share if k != "relax"), key=share.get)
    exp_p, exp_m = sim.export_state()
    bbar = float(np.clip(exp_p["n_active_interactions"], 0, 8).mean())
    finite = bool(np.isfinite(exp_p["pos"][(exp_p["flags"] & 1) != 0]).all()
                  and np.isfinite(exp_m["pos"][(exp_m["flags"] & 1) != 0]).all())
    peak, peak_kind = _measured_peaks()
    alg = algorithmic_bytes(dom, N, Nm, S, bbar)
    achieved = alg / (phase_ms[dom] / 1e3) / 1e9
    step_bytes = step_algorithmic_bytes(cfg, bbar)
    step_achieved = step_bytes / (ms_per_step / 1e3) / 1e9
    traffic = measured_traffic(dom, args.workload) if args.fraction == 1.0 else None
    # The metabolic relaxation's neighbour data moves through the SM's L1 /
    # shared-memory data pipe: a position and a velocity (2 x 16 B) and a
    # 4-byte list entry per pair, the item's own 3 records and its output.
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_hz = (clocks.summary().get("sm_mhz") or 2070.0) * 1e6
    l1_peak = sms * 128 * sm_hz / 1e9
    l1_bytes = pairs[1] * 36 + Nm * 64 if pairs[1] >= 0 else None
    l1 = None if l1_bytes is None else {
        "kernel": "relax_metab", "pairs_per_launch": pairs[1], "bytes_per_launch": l1_bytes,
        "achieved": l1_bytes / (phase_ms["relax_metab"] / 1e3) / 1e9, "peak": l1_peak, "unit": "GB/s",
        "frac": l1_bytes / (phase_ms["relax_metab"] / 1e3) / 1e9 / l1_peak,
        "peak_is": f"{sms} SMs x 128 B/clock at the sampled SM clock"}

    # end to end through the C ABI with host buffers
    sim2 = native.Simulation(cfg, types, rules)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim2.load_state_ptr(ctypes.c_void_p(p_host.data_ptr()), N, ctypes.c_void_p(m_host.data_ptr()), Nm, 0, N)
    t_load = time.perf_counter()
    sim2.prepare()
    sim2.sync()
    t_prep = time.perf_counter()
    ticket = -1
    for k in range(args.steps):
        sim2.step(1)
        ticket = sim2.reduce_frame_async_ptr(ctypes.c_void_p(rp_host[k % 2].data_ptr()),
                                             ctypes.c_void_p(rm_host[k % 2].data_ptr()))
    sim2.frame_wait(ticket)
    sim2.sync()
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"load_ms": 1e3 * (t_load - t0), "prepare_ms": 1e3 * (t_prep - t_load),
                 "steps_with_frames_ms": 1e3 * (t0 + e2e_s - t_prep)}
    sim2.close()
    e2e_rate, _ = aggregate_replicas(items, args.steps, e2e_s, device="cuda")
    e2e = {"value": e2e_rate, "unit": UNIT,
           "h2d_bytes_per_step": int((p.nbytes + m.nbytes) / args.steps),
           "d2h_bytes_per_step": int(rp_host[0].numel() + rm_host[0].numel()),
           "includes": "sc_load_state of the initial AoS state + sc_prepare, then per step sc_step + "
                       "sc_reduce_frame_async into pinned host memory (the copy overlaps the next step); "
                       "ends when the last frame has landed",
           "parts": e2e_parts}
    sim.close()
    batched = batched_sample(args, native, torch) if args.batch_replicas > 0 and world == 1 else None
    served = serving_sample(args) if args.serve_requests > 0 and world == 1 else None
    vesicle = vesicle_sample(args, native, torch) if args.vesicle_scale > 0 and world == 1 else None
    ref_cuda = reference_cuda_sample(args, native, torch) if args.ref_steps > 0 and world == 1 else None

    line = None
    if rank == 0:
        cpu_rate, cpu_threads, cpu_desc = cpu_sample(args, reps=2) if not args.no_cpu else (None, 0, "skipped")
        cpu_one = cpu_single_core(args) if not args.no_cpu else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded; no dataset in the reference)",
            "config": {"workload": args.workload if args.fraction == 1.0
                       else f"{args.workload} (sub-box, {args.fraction:g} of its volume)",
                       "particles": N, "metabolic_particles": Nm,
                       "box_nm": cfg.sim_size, "cell_nm": cfg.grid_cell_size, "species": S,
                       "sub_iterations": [cfg.noise_coordination_steps, cfg.relaxation_steps,
                                          cfg.metabolite_diffusion_steps],
                       "l2": "inputs larger than L2 (state of several GB)",
                       "complexify": "pair claim, A + B bind at probability %g per step"
                                     % scenes.WORKLOAD_BIND_PROBABILITY,
                       "metabolic_pairs": "4-byte entries" if args.metabolic_pairs == 0 else "16-byte entries",
                       "parallelism": f"replicas x{world}"},
            "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": alg, "launch_ms": phase_ms[dom]},
            "step_roofline": {"bound": "hbm", "achieved": step_achieved, "peak": peak, "unit": "GB/s",
                              "frac": step_achieved / peak, "algorithmic_bytes_per_step": step_bytes},
            "l1_roofline": l1,
            "pairs_per_list": {"particle": pairs[0], "metabolic": pairs[1], "lipid_metabolic": pairs[2],
                               "diffusion": pairs[3]},
            "phase_ms_per_launch": phase_ms, "phase_share_of_step": share,
            "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                             "sample": cpu_desc, "single_core": cpu_one},
            "state_finite": finite, "bonds_per_particle": bbar,
            "device_bytes": {"sim": footprint, "per_item": footprint / (N + Nm),
                             "note": "sc_device_bytes after the warm-up steps: state, lists and pools"},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
            "batched": batched,
            "serving": served,
            "vesicle": vesicle,
            "reference_cuda": ref_cuda,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_large", choices=sorted(scenes.WORKLOADS))
    ap.add_argument("--cpu-fraction", type=float, default=0.25,
                    help="volume fraction of the workload the CPU oracle steps (its timed sample)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-replicas", type=int, default=512,
                    help="replica cells in the batched sample (0: skip it)")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--serve-requests", type=int, default=32,
                    help="requests of the serving sample's latency runs (0: skip the serving sample)")
    ap.add_argument("--serve-saturated", type=int, default=240,
                    help="requests of the serving sample's saturated run (enough that the 160 GB budget binds)")
    ap.add_argument("--serve-horizon", type=int, default=150, help="longest request horizon (steps)")
    ap.add_argument("--vesicle-scale", type=float, default=1.0,
                    help="count scale of the vesicle sample (0: skip it)")
    ap.add_argument("--vesicle-steps", type=int, default=100)
    ap.add_argument("--vesicle-replica-steps", type=int, default=25,
                    help="steps of each of the four vesicle replicas")
    ap.add_argument("--metabolic-pairs", type=int, default=1, choices=[0, 1],
                    help="metabolic relaxation pairs: 0 4-byte entries (geometry per sub-iteration), "
                         "1 16-byte entries with the geometry frozen per step")
    ap.add_argument("--ref-steps", type=int, default=4,
                    help="steps of the reference's CUDA step timed beside this build's (0: skip)")
    ap.add_argument("--fraction", type=float, default=1.0,
                    help="run a same-density sub-box of this volume fraction (small cases for profiling)")
    ap.add_argument("--cpu-small-full", action="store_true",
                    help="only run the small workload in full (200 steps) on the CPU oracle and print its line")
    args = ap.parse_args()
    if args.cpu_small_full:
        print(json.dumps(cpu_small_full(args)))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
