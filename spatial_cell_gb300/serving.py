"""Continuous-batching request loop over independent simulations.

A request asks for a simulation cell at the small workload's number density
(seed, particle count, horizon in steps, lipid / dummy / A / B mix).  The
server admits requests in arrival order against a device-memory budget,
keeps every admitted simulation resident on the GPU on its own CUDA stream,
and gives each one its next step (a captured graph) as soon as its previous
step has finished, so the steps of all admitted requests overlap on the
device.  A request that reaches its horizon is handed its final frame (the
frames.dat payload) and retired, freeing its memory for the requests still
waiting; requests that arrive while others run are admitted as memory frees
up.  Each simulation is independent, so a request's result does not depend
on the mix it ran in.
"""
import dataclasses
import time

import numpy as np

from . import abi, native, scenes

# Device bytes per item of a simulation: state (two buffers of every field)
# and pair lists, from the allocation in sc_create; an upper bound used for
# admission.
BYTES_PER_PARTICLE = 1800
BYTES_PER_METABOLIC = 2200


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the run
    seed: int
    n: int
    horizon: int
    mix: tuple = (0.4, 0.4, 0.1, 0.1)

    @property
    def nm(self):
        return 2 * self.n

    @property
    def bytes(self):
        return self.n * BYTES_PER_PARTICLE + self.nm * BYTES_PER_METABOLIC

    def config(self):
        """The request's cell: the small workload's density and physics."""
        box = float(200.0 * (self.n / 65536.0) ** (1.0 / 3.0))
        return scenes.measured_config("plain_small", num_particles=self.n, num_metabolic_particles=self.nm,
                                      sim_size=box, seed=self.seed)

    def start(self):
        """A simulation of the request, its scene generated on the device."""
        sim = native.Simulation(self.config(), scenes.baseline_types(), scenes.workload_rules())
        sim.generate_uniform(self.n, self.nm, (scenes.LIPID, scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B), self.mix,
                             self.seed)
        sim.prepare()
        return sim


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    frame: tuple  # (reduced particles, reduced metabolic)

    @property
    def latency(self):
        return self.finished - self.arrival


def poisson_requests(count, rate, seed=4, n_lo=4096, n_hi=1048576, h_lo=100, h_hi=5000):
    """`count` requests arriving as a Poisson stream of `rate` per second:
    particle counts log-uniform in [n_lo, n_hi], horizons uniform in
    [h_lo, h_hi] steps, mix ~ Dirichlet(1, 1, 1, 1)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for k in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        h = int(rng.integers(h_lo, h_hi + 1))
        mix = tuple(float(x) for x in rng.dirichlet([1.0, 1.0, 1.0, 1.0]))
        out.append(Request(k, float(t[k]), seed * 100000 + k, n, h, mix))
    return out


class Server:
    """Admits, steps and retires requests; `run` serves a list of requests
    whose arrival times are relative to its start."""

    def __init__(self, budget_bytes):
        self.budget = budget_bytes

    def run(self, requests, clock=time.perf_counter):
        waiting = sorted(requests, key=lambda r: r.arrival)
        active = []  # (request, sim, admitted time, steps done)
        results = []
        used = 0
        t0 = clock()
        while waiting or active:
            now = clock() - t0
            # admit arrived requests in order while memory allows
            while waiting and waiting[0].arrival <= now and used + waiting[0].bytes <= self.budget:
                r = waiting.pop(0)
                sim = r.start()
                used += r.bytes
                active.append([r, sim, clock() - t0, 0])
            if not active:
                if waiting:  # idle until the next arrival
                    time.sleep(max(0.0, min(waiting[0].arrival - now, 0.01)))
                continue
            # Every request whose previous step has finished gets its next one
            # (each on its own stream, so the steps of all requests overlap);
            # one whose horizon is reached is handed its frame and retired.
            still = []
            progressed = False
            for a in active:
                r, sim, adm, steps = a
                if not sim.idle():
                    still.append(a)
                    continue
                progressed = True
                if steps >= r.horizon:
                    frame = sim.reduce_frame()
                    results.append(Result(r.rid, r.arrival, adm, clock() - t0, steps, frame))
                    sim.close()
                    used -= r.bytes
                    continue
                sim.step(1)
                a[3] += 1
                still.append(a)
            active = still
            if not progressed:
                time.sleep(20e-6)
        return results


def serve_alone(request):
    """The request run by itself: its final frame."""
    res = Server(budget_bytes=1 << 62).run([dataclasses.replace(request, arrival=0.0)])
    return res[0].frame


def percentiles(results):
    lat = np.array([r.latency for r in results])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))


def throughput(results, requests):
    by_id = {r.rid: r for r in requests}
    work = sum((by_id[x.rid].n + by_id[x.rid].nm) * x.steps for x in results)
    span = max(x.finished for x in results) - min(x.arrival for x in results)
    return work / span


__all__ = ["Request", "Result", "Server", "poisson_requests", "serve_alone", "percentiles", "throughput", "abi"]
