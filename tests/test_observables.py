"""FP64 observables (sc_observe, sc_mark_positions, sc_pair_histogram).

CPU tests pin the host oracle (oracle/observables.py) on hand-built cases;
the GPU tests compare the device reductions with the oracle evaluated on the
CPU engine's own trajectory (the two trajectories are bit-identical, so the
observables agree to double-precision rounding and the histograms exactly)."""
import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes
from oracle import observables as obs


def _pair(pos_a, pos_b, types=(scenes.DUMMY, scenes.DUMMY)):
    p = np.zeros(2, abi.PARTICLE_DTYPE)
    p["id"] = [0, 1]
    p["flags"] = abi.PARTICLE_FLAG_ACTIVE
    p["type"] = types
    p["pos"] = [pos_a, pos_b]
    return p


def test_oracle_pair_histogram_minimum_image():
    # 1.5 nm apart across the periodic face of a 20 nm box
    p = _pair((0.25, 5.0, 5.0), (18.75, 5.0, 5.0))
    h = obs.pair_histogram(p, -1, -1, 3.0, 6, 20.0, True)
    assert h.tolist() == [0, 0, 0, 2, 0, 0]  # both orders, bin [1.5, 2.0)
    assert obs.pair_histogram(p, -1, -1, 3.0, 6, 20.0, False).sum() == 0  # walls: 18.5 apart
    # typed: only (A, B) ordered pairs
    q = _pair((1.0, 1.0, 1.0), (2.0, 1.0, 1.0), types=(scenes.TYPE_A, scenes.TYPE_B))
    assert obs.pair_histogram(q, scenes.TYPE_A, scenes.TYPE_B, 2.0, 4, 20.0, False).tolist() == [0, 0, 1, 0]


def test_oracle_msd_and_counts():
    p = _pair((1.0, 1.0, 1.0), (5.0, 5.0, 5.0))
    o = obs.mark(p)
    p["pos"][0] = (2.0, 1.0, 1.0)   # moved 1
    p["pos"][1] = (5.0, 7.0, 5.0)   # moved 2
    p["velocity"][1] = (0.0, 3.0, 4.0)
    r = obs.observe(p, o, 20.0, False)
    assert r["msd"] == pytest.approx(2.5) and r["msd_items"] == 2 and r["active"] == 2
    assert r["mean_v2"] == pytest.approx(12.5)
    p["pos"][1] = (5.0, 5.0, 19.5)  # 5.5 forward through the face = 5.5 back by the minimum image
    assert obs.observe(p, o, 20.0, True)["msd"] == pytest.approx((1.0 + 5.5 ** 2) / 2)


def _engines(product, seed=21, periodic=1):
    from oracle.engine import OracleEngine
    cfg, types, rules, p, m, nid = scenes.test_scene(seed, n=900, nm=1800, box=42.0, periodic=periodic)
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=nid)
        e.prepare()
    return cfg, gpu, cpu


def _check(cfg, gpu, cpu, origins, what):
    pc, mc = cpu.export_state()
    got = gpu.observe()
    for k, (recs, extra) in enumerate(((pc, dict(bonds=True)), (mc, dict(species=cfg.num_metabolites)))):
        ref = obs.observe(recs, origins[k], cfg.sim_size, bool(cfg.periodic), **extra)
        assert got["msd_items"][k] == ref["msd_items"] and got["active"][k] == ref["active"], what
        # the walled test scene stacks items on the walls, where the reference's normalize(0) gives NaN
        # velocities: NaN on one side must be NaN on the other
        assert np.isclose(got["msd"][k], ref["msd"], rtol=1e-12, atol=1e-12, equal_nan=True), what
        assert np.isclose(got["mean_v2"][k], ref["mean_v2"], rtol=1e-12, atol=1e-12, equal_nan=True), what
    assert got["bond_slots"] == obs.observe(pc, None, cfg.sim_size, bool(cfg.periodic), bonds=True)["bond_slots"]
    ref_m = obs.observe(mc, None, cfg.sim_size, bool(cfg.periodic), species=cfg.num_metabolites)["metabolites"]
    assert np.allclose(got["metabolites"][:cfg.num_metabolites], ref_m, rtol=1e-12, atol=1e-9, equal_nan=True), what


@pytest.mark.gpu
@pytest.mark.parametrize("periodic", [1, 0])
def test_device_observables_follow_the_oracle(product, periodic):
    cfg, gpu, cpu = _engines(product, periodic=periodic)
    gpu.mark_positions()
    pc, mc = cpu.export_state()
    origins = (obs.mark(pc), obs.mark(mc))
    _check(cfg, gpu, cpu, origins, "at the mark")
    for e in (gpu, cpu):
        e.step(40)
    _check(cfg, gpu, cpu, origins, "40 steps after the mark")
    assert gpu.observe()["msd"][1] > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("types", [(-1, -1), (scenes.LIPID, scenes.LIPID), (scenes.TYPE_A, scenes.TYPE_B)])
def test_device_pair_histogram_matches_the_oracle(product, types):
    cfg, gpu, cpu = _engines(product, seed=22)
    for e in (gpu, cpu):
        e.step(3)
    h = gpu.pair_histogram(types[0], types[1], 6.0, 24)
    pc, _ = cpu.export_state()
    ref = obs.pair_histogram(pc, types[0], types[1], 6.0, 24, cfg.sim_size, bool(cfg.periodic))
    assert h.tolist() == ref.tolist()
    # the histogram sorted the particles into their cells; the trajectory is unchanged
    for e in (gpu, cpu):
        e.step(2)
    from tests.helpers import assert_same_state
    assert_same_state(gpu.export_state(), cpu.export_state(), species=cfg.num_metabolites,
                      what="steps after a histogram")


@pytest.mark.gpu
def test_pair_histogram_refuses_radius_beyond_a_cell(product):
    from spatial_cell_gb300.native import ScError
    cfg, gpu, _ = _engines(product)
    with pytest.raises(ScError):
        gpu.pair_histogram(-1, -1, cfg.grid_cell_size * 1.5, 8)


@pytest.mark.gpu
def test_ensemble_msd_and_rdf_after_1000_steps(product):
    """The small workload's physics (1,024 particles, 2,048 metabolic items,
    periodic 50 nm cube) for 1000 steps on the device and on the CPU oracle:
    the device's FP64 MSD and pair-distance histogram stay within 1 % of the
    host oracle's (they agree to rounding, the trajectories being identical)."""
    from oracle.engine import OracleEngine
    n, nm = 1024, 2048
    cfg = scenes.workload_config("plain_small", num_particles=n, num_metabolic_particles=nm,
                                 sim_size=200.0 * (n / 65536.0) ** (1.0 / 3.0), seed=3)
    rng = np.random.default_rng(3)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, cfg.sim_size, types)
    m = scenes.uniform_metabolic(rng, nm, cfg.sim_size, types, cfg.num_metabolites)
    gpu = product.Simulation(cfg, types, rules)
    cpu = OracleEngine("port", cfg, types, rules)
    for e in (gpu, cpu):
        e.load_state(p, m, step=0, next_particle_id=n)
        e.prepare()
    gpu.mark_positions()
    pc, mc = cpu.export_state()
    origins = (obs.mark(pc), obs.mark(mc))
    for e in (gpu, cpu):
        e.step(1000)
    got = gpu.observe()
    pc, mc = cpu.export_state()
    for k, recs in enumerate((pc, mc)):
        ref = obs.observe(recs, origins[k], cfg.sim_size, True)
        assert abs(got["msd"][k] - ref["msd"]) <= 0.01 * ref["msd"]
        assert got["msd"][k] == pytest.approx(ref["msd"], rel=1e-12)
    h = gpu.pair_histogram(-1, -1, 6.0, 24).astype(np.float64)
    ref_h = obs.pair_histogram(pc, -1, -1, 6.0, 24, cfg.sim_size, True).astype(np.float64)
    big = ref_h >= 100
    assert (np.abs(h[big] - ref_h[big]) <= 0.01 * ref_h[big]).all()
    assert h.tolist() == ref_h.tolist()
