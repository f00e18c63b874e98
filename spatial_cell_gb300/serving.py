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

# Device bytes per item of a request's simulation (state, two buffers of
# every field, and pair lists as sc_create and sc_prepare size them at this
# density), used to decide admission; once admitted, a request counts against
# the budget with what its sim holds (sc_device_bytes).
BYTES_PER_PARTICLE = 1400
BYTES_PER_METABOLIC = 1700


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


class FrameStream:
    """A request's frames streamed to the host while it runs: every
    `every` steps (and at the horizon) the frames.dat payload of its state is
    reduced on the device and copied into one of two pinned host slots while
    the next steps run (sc_reduce_frame_async); `deliver(rid, step, frame)`
    receives each frame once it has landed (the default keeps the last)."""

    def __init__(self, sim, n, nm, every, deliver=None):
        self.sim, self.every, self.deliver = sim, every, deliver
        self.rp = self.rm = None  # pinned slots, taken at the first frame
        self.n, self.nm = n, nm
        self.pending = []  # (ticket, slot, step)
        self.count = 0
        self.bytes = 0
        self.last = None

    def _land(self, rid, keep):
        t, slot, step = self.pending.pop(0)
        self.sim.frame_wait(t)
        self.count += 1
        self.bytes += self.rp[slot].numel() + self.rm[slot].numel()
        if self.deliver or keep:
            frame = (self.rp[slot].numpy()[:self.n * abi.REDUCED_DTYPE.itemsize].copy().view(abi.REDUCED_DTYPE),
                     self.rm[slot].numpy()[:self.nm * abi.REDUCED_METABOLIC_DTYPE.itemsize].copy()
                     .view(abi.REDUCED_METABOLIC_DTYPE))
            if self.deliver:
                self.deliver(rid, step, frame)
            self.last = frame

    def push(self, rid, step, final=False):
        """Streams the frame of the state after `step` steps (when due)."""
        import ctypes
        if not final and (self.every <= 0 or step % self.every):
            return
        if self.rp is None:
            import torch
            self.rp = [torch.empty(max(self.n, 1) * abi.REDUCED_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
                       for _ in range(2)]
            self.rm = [torch.empty(max(self.nm, 1) * abi.REDUCED_METABOLIC_DTYPE.itemsize, dtype=torch.uint8,
                                   pin_memory=True) for _ in range(2)]
        if len(self.pending) == 2:  # both slots in flight: the oldest lands first
            self._land(rid, False)
        slot = self.count + len(self.pending)
        slot &= 1
        t = self.sim.reduce_frame_async_ptr(ctypes.c_void_p(self.rp[slot].data_ptr()),
                                            ctypes.c_void_p(self.rm[slot].data_ptr()))
        self.pending.append((t, slot, step))

    def finish(self, rid):
        while self.pending:
            self._land(rid, not self.pending[1:])
        return self.last


class Server:
    """Admits, steps and retires requests; `run` serves a list of requests
    whose arrival times are relative to its start.

    Requests are admitted in arrival order while the device memory they will
    hold fits the budget.  Each admitted request is a sim of its own on its
    own stream; it gets its next step as soon as its previous one has
    finished on the device -- the library queues a completion notice for it
    (sc_set_notify) and the loop blocks on the notice queue
    (sc_wait_notices) until some request is ready or the next request
    arrives.  Frames of every request stream to the host every
    `frame_every` steps and at its horizon (FrameStream); a request whose
    horizon is reached is retired with its last frame, freeing its memory."""

    def __init__(self, budget_bytes, frame_every=0, deliver=None):
        self.budget = budget_bytes
        self.frame_every = frame_every
        self.deliver = deliver
        self.frames = 0
        self.frame_bytes = 0

    def run(self, requests, clock=time.perf_counter):
        waiting = sorted(requests, key=lambda r: r.arrival)
        active = {}  # rid -> [request, sim, admitted time, steps done, frames]
        ready = []
        results = []
        used = 0
        t0 = clock()
        while waiting or active:
            now = clock() - t0
            # admit arrived requests in order while memory allows
            while waiting and waiting[0].arrival <= now and used + waiting[0].bytes <= self.budget:
                r = waiting.pop(0)
                sim = r.start()
                sim.set_notify(r.rid)
                held = sim.device_bytes()  # what it holds, once its pools are sized (sc_prepare)
                used += held
                fs = FrameStream(sim, r.n, r.nm, self.frame_every, self.deliver)
                active[r.rid] = [r, sim, clock() - t0, 0, fs, held]
                ready.append(r.rid)
            for rid in ready:
                a = active[rid]
                r, sim, adm, steps, fs, held = a
                if steps >= r.horizon:
                    frame = fs.finish(rid) if fs.count + len(fs.pending) else None
                    if frame is None:
                        fs.push(rid, steps, final=True)
                        frame = fs.finish(rid)
                    self.frames += fs.count
                    self.frame_bytes += fs.bytes
                    results.append(Result(r.rid, r.arrival, adm, clock() - t0, steps, frame))
                    sim.close()
                    used -= held
                    del active[rid]
                    continue
                sim.step(1)
                a[3] += 1
                fs.push(rid, a[3], final=a[3] == r.horizon)
            # block until a request's step has finished, or until the next
            # arrival (a request that has arrived but does not fit waits for a
            # retirement, which a notice announces)
            ahead = waiting[0].arrival - (clock() - t0) if waiting else -1.0
            if active:
                ready = native.wait_notices(timeout_ms=int(1e3 * ahead) + 1 if ahead > 0 else -1)
            else:
                ready = []
                if ahead > 0:
                    time.sleep(ahead)
        return results


def serve_alone(request):
    """The request run by itself: its final frame."""
    res = Server(budget_bytes=1 << 62).run([dataclasses.replace(request, arrival=0.0)])
    return res[0].frame


def saturated(requests):
    """The same requests all arriving at once (arrivals faster than any
    capacity): the server's throughput when the budget, not the arrivals,
    limits what runs."""
    return [dataclasses.replace(r, arrival=0.0) for r in requests]


def percentiles(results):
    lat = np.array([r.latency for r in results])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))


def throughput(results, requests):
    by_id = {r.rid: r for r in requests}
    work = sum((by_id[x.rid].n + by_id[x.rid].nm) * x.steps for x in results)
    span = max(x.finished for x in results) - min(x.arrival for x in results)
    return work / span


__all__ = ["Request", "Result", "Server", "FrameStream", "poisson_requests", "serve_alone", "saturated",
           "percentiles", "throughput", "abi"]
