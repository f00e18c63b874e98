"""The allocation-free cell sort, sc_sort_cells_static, through the C ABI.

It exists for callers that cannot let the library allocate device memory
(a framework that owns the GPU's memory pool, a loop that cannot absorb
cudaMalloc's synchronisation).  Its result must equal a sim's own sort of the
same state: the sort permutation and the cell-start table are integer
results, so the comparison is exact.  Two calls in a row check that the
shared static scratch is cleared between calls.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

MAX_ITEMS = 1 << 18


def _soa(p, cap):
    """float4 (x, y, z, radius) and int4 (id, type, flags, hydrophobic) of a
    capacity-sized state whose first len(p) items are p."""
    pos = np.zeros((cap, 4), np.float32)
    info = np.zeros((cap, 4), np.int32)
    n = len(p)
    pos[:n, :3] = p["pos"]
    pos[:n, 3] = p["radius"]
    info[:n, 0] = p["id"]
    info[:n, 1] = p["type"]
    info[:n, 2] = p["flags"]
    info[:n, 3] = p["hydrophobic"]
    return pos, info


def _ranges(cell_start, cells):
    cs = cell_start.astype(np.int64)
    start, end = cs[:-1], cs[1:]
    empty = start == end
    r = np.zeros(2 * cells, np.uint32)
    r[0::2] = np.where(empty, 0, start)
    r[1::2] = np.where(empty, 0, end)
    return r


def _scene(kind):
    if kind == "mixed":
        return scenes.test_scene(21, n=3000, nm=64, box=50.0)
    n = 200000
    box = float(635.0 * (n / 2097152) ** (1.0 / 3.0))
    cfg = scenes.workload_config("plain_large", num_particles=n, num_metabolic_particles=64, sim_size=box, seed=4)
    rng = np.random.default_rng(4)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, box, types)
    p["flags"][rng.random(n) < 0.01] = 0   # a few inactive items in the middle
    m = scenes.uniform_metabolic(rng, 64, box, types, cfg.num_metabolites)
    return cfg, types, rules, p, m, n


@pytest.mark.parametrize("kind", ["mixed", "uniform"])
def test_static_sort_matches_sim_sort(product, kind):
    import torch
    cfg, types, rules, p, m, nid = _scene(kind)
    sim = product.Simulation(cfg, types, rules)
    sim.load_state(p, m, next_particle_id=nid)
    sim.run_phase(abi.PHASE_SORT_PARTICLES)
    ranges_ref, perm_ref = sim.export_grid(0)
    sim.close()

    cap = cfg.num_particles
    cells = abi.grid_dims(cfg)[2]
    assert cap <= MAX_ITEMS
    pos, info = _soa(p, cap)
    dpos = torch.from_numpy(pos).cuda()
    dinfo = torch.from_numpy(info).cuda()
    stream = torch.cuda.current_stream()
    L = product.lib()
    for call in range(2):
        dperm = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        dcs = torch.full((cells + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.sc_sort_cells_static(ctypes.byref(cfg), ctypes.c_void_p(dpos.data_ptr()),
                                    ctypes.c_void_p(dinfo.data_ptr()), cap, ctypes.c_void_p(dperm.data_ptr()),
                                    ctypes.c_void_p(dcs.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, f"call {call}: status {rc}"
        perm = dperm.cpu().numpy().view(np.uint32)
        cs = dcs.cpu().numpy().view(np.uint32)
        assert np.array_equal(perm, perm_ref), f"call {call}: permutation differs from the sim's sort"
        assert np.array_equal(_ranges(cs, cells), ranges_ref), f"call {call}: cell ranges differ"


def _static_sort(product, cfg, pos, info, n, cells):
    """perm, cell_start of one call on torch's current stream."""
    import torch
    dpos = torch.from_numpy(pos).cuda()
    dinfo = torch.from_numpy(info).cuda()
    dperm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    dcs = torch.full((cells + 1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = product.lib().sc_sort_cells_static(ctypes.byref(cfg), ctypes.c_void_p(dpos.data_ptr()),
                                            ctypes.c_void_p(dinfo.data_ptr()), n, ctypes.c_void_p(dperm.data_ptr()),
                                            ctypes.c_void_p(dcs.data_ptr()),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, f"status {rc}"
    return dperm.cpu().numpy().view(np.uint32)[:n], dcs.cpu().numpy().view(np.uint32)


def test_static_sort_of_no_items(product):
    """n = 0: every cell starts (and ends) at slot 0."""
    cfg = scenes.workload_config("plain_small", num_particles=16)
    cells = abi.grid_dims(cfg)[2]
    for _ in range(2):
        _, cs = _static_sort(product, cfg, np.zeros((1, 4), np.float32), np.zeros((1, 4), np.int32), 0, cells)
        assert not cs.any()


def test_static_sort_at_its_capacity(product):
    """n = 262,144, the array's limit: the last look-back tile is in use, and
    items of the last tile sit in cells of their own.  Compared with a sim's
    sort and with a stable argsort of the cell keys in numpy, on two calls."""
    n = MAX_ITEMS
    box = float(635.0 * (n / 2097152) ** (1.0 / 3.0))
    cfg = scenes.workload_config("plain_large", num_particles=n, num_metabolic_particles=64, sim_size=box, seed=5,
                                 periodic=0)  # the reference's key: min(coord / cell, cells - 1) per axis
    rng = np.random.default_rng(5)
    types, rules = scenes.baseline_types(), scenes.baseline_rules()
    p = scenes.uniform_particles(rng, n, box, types)
    p["pos"][-64:] = np.float32(box - 0.01)           # the last tile's tail in the last cell
    p["flags"][rng.random(n) < 0.01] = 0
    m = scenes.uniform_metabolic(rng, 64, box, types, cfg.num_metabolites)
    sim = product.Simulation(cfg, types, rules)
    sim.load_state(p, m, next_particle_id=n)
    sim.run_phase(abi.PHASE_SORT_PARTICLES)
    ranges_ref, perm_ref = sim.export_grid(0)
    sim.close()
    ngrid, bits, cells = abi.grid_dims(cfg)
    idx = np.minimum((p["pos"] / np.float32(cfg.grid_cell_size)).astype(np.uint32), ngrid - 1)
    keys = (idx[:, 0] << np.uint32(2 * bits)) | (idx[:, 1] << np.uint32(bits)) | idx[:, 2]
    keys = np.where((p["flags"] & 1) != 0, keys, np.uint32(0xFFFFFFFF))
    perm_np = np.argsort(keys, kind="stable").astype(np.uint32)
    assert np.array_equal(perm_np, perm_ref)
    pos, info = _soa(p, n)
    for call in range(2):
        perm, cs = _static_sort(product, cfg, pos, info, n, cells)
        assert np.array_equal(perm, perm_ref), f"call {call}: permutation differs"
        assert np.array_equal(_ranges(cs, cells), ranges_ref), f"call {call}: cell ranges differ"


def test_static_sort_rejects_more_than_its_capacity(product):
    import torch
    cfg = scenes.workload_config("plain_small", num_particles=MAX_ITEMS + 1)
    cells = abi.grid_dims(cfg)[2]
    small = torch.zeros(16, dtype=torch.int32, device="cuda")
    cs = torch.zeros(cells + 1, dtype=torch.int32, device="cuda")
    ptr = ctypes.c_void_p(small.data_ptr())
    rc = product.lib().sc_sort_cells_static(ctypes.byref(cfg), ptr, ptr, MAX_ITEMS + 1, ptr,
                                            ctypes.c_void_p(cs.data_ptr()), None)
    assert rc == -1  # SC_E_INVALID, nothing launched
