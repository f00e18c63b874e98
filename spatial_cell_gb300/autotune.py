"""Launch-configuration autotuner for replica cells.

For a cell of a given size the step's speed depends on choices that do not
change what is simulated beyond the floating-point order of the neighbour
sums: the grid cell size (any size at least the interaction and diffusion
ranges keeps every pair in the 27-cell neighbourhood), whether the particle
work classes run on three streams, and whether the metabolic sweep runs on
shared-memory tiles.  The tuner times every candidate on a device-generated
scene of the cell's size and mix and returns the fastest; its choice is then
used for every replica of that size class.  Results at the chosen settings
are checked against the oracle like any other configuration (the oracle
takes the same config).  Every choice is a field of the sim's sc_config, so
tuning touches no process-wide state.
"""
import itertools
import time

from . import abi, native, scenes


def candidates(cfg, cells=(6.0, 7.0, 8.0), fork=(0, 1), tiles=(0, 1)):
    """(cell size, fork, tiles) triples valid for cfg: cells no smaller than
    the interaction and diffusion ranges, and leaving a periodic box at
    least three cells wide."""
    lo = max(cfg.max_interaction_distance, cfg.max_diffusion_distance)
    out = []
    for c, f, t in itertools.product(cells, fork, tiles):
        if c < lo:
            continue
        if cfg.periodic and cfg.sim_size / c < 3.0:
            continue
        out.append((float(c), int(f), int(t)))
    return out


def time_candidate(cfg, types, rules, kinds, fractions, seed, steps, cell, fork, tiles):
    """Seconds per step of one candidate on a device-generated scene."""
    c = apply(cfg, (cell, fork, tiles))
    sim = native.Simulation(c, types, rules)
    try:
        sim.generate_uniform(c.num_particles, c.num_metabolic_particles, kinds, fractions, seed)
        sim.prepare()
        sim.step(1)  # captures the step graph
        sim.sync()
        t0 = time.perf_counter()
        sim.step(steps)
        sim.sync()
        return (time.perf_counter() - t0) / steps
    finally:
        sim.close()


def tune(cfg, types=None, rules=None, kinds=(scenes.LIPID, scenes.DUMMY, scenes.TYPE_A, scenes.TYPE_B),
         fractions=(0.4, 0.4, 0.1, 0.1), seed=1, steps=3, timer=None, **cand):
    """The fastest (cell size, fork, tiles) for cfg and every candidate's time:
    returns (best, {candidate: seconds per step}).  `timer` replaces the
    device timing (tests)."""
    types = scenes.baseline_types() if types is None else types
    rules = scenes.baseline_rules() if rules is None else rules
    timer = timer or (lambda cell, fork, tiles: time_candidate(cfg, types, rules, kinds, fractions, seed, steps,
                                                               cell, fork, tiles))
    times = {c: timer(*c) for c in candidates(cfg, **cand)}
    if not times:
        raise ValueError("no valid candidate for this config")
    return min(times, key=lambda c: (times[c], c)), times


def apply(cfg, choice):
    """cfg with the chosen (cell size, fork, tiles): fork 1 runs the particle
    work classes on three streams, 0 on the sim's stream."""
    d = cfg.as_dict()
    d["grid_cell_size"] = choice[0]
    d["class_streams"] = 3 if choice[1] else 1
    d["tiles"] = int(choice[2])
    return abi.make_config(**d)


def batch_cells(cfg, cells=(6.0, 7.0, 8.0)):
    """Grid cell sizes to try for a batch of replicas with cfg's physics (the
    smallest replica's box is checked by sc_create_batch)."""
    lo = max(cfg.max_interaction_distance, cfg.max_diffusion_distance)
    return [float(c) for c in cells if c >= lo]
