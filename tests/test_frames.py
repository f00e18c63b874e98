"""Streamed frames (sc_reduce_frame_async / sc_frame_wait) carry the same
bytes as the synchronous sc_reduce_frame of the same states, with more
frames in flight than staging slots."""
import ctypes

import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_streamed_frames_equal_synchronous_frames(product):
    torch = pytest.importorskip("torch")
    cfg, types, rules, p, m, nid = scenes.test_scene(21, n=900, nm=1800, box=42.0, periodic=1)
    steps = 5
    sims = []
    for _ in range(2):
        s = product.Simulation(cfg, types, rules)
        s.load_state(p, m, next_particle_id=nid)
        s.prepare()
        sims.append(s)
    nbp = cfg.num_particles * abi.REDUCED_DTYPE.itemsize
    nbm = cfg.num_metabolic_particles * abi.REDUCED_METABOLIC_DTYPE.itemsize
    hp = [torch.zeros(nbp, dtype=torch.uint8, pin_memory=True) for _ in range(steps)]
    hm = [torch.zeros(nbm, dtype=torch.uint8, pin_memory=True) for _ in range(steps)]
    tickets = []
    for k in range(steps):
        sims[0].step(1)
        tickets.append(sims[0].reduce_frame_async_ptr(ctypes.c_void_p(hp[k].data_ptr()),
                                                      ctypes.c_void_p(hm[k].data_ptr())))
    assert tickets == list(range(steps))
    sims[0].frame_wait(tickets[1])
    sims[0].frame_wait(tickets[-1])
    for k in range(steps):
        sims[1].step(1)
        rp, rm = sims[1].reduce_frame()
        assert hp[k].numpy().tobytes() == rp.tobytes(), f"particle frame {k} differs"
        assert hm[k].numpy().tobytes() == rm.tobytes(), f"metabolic frame {k} differs"
    # the synchronous form still works after streamed frames
    rp0, rm0 = sims[0].reduce_frame()
    assert rp0.tobytes() == rp.tobytes() and rm0.tobytes() == rm.tobytes()
    for s in sims:
        s.close()


def test_checkpoint_resume_continues_bit_for_bit(product, tmp_path):
    """Four steps straight == two steps, checkpoint, a new sim resumes, two
    more steps (same bytes of the whole state and the same counters)."""
    scene = scenes.test_scene(23, n=900, nm=1800, box=42.0, periodic=1)
    cfg, types, rules, p, m, nid = scene
    a = product.Simulation(cfg, types, rules)
    a.load_state(p, m, next_particle_id=nid)
    a.prepare()
    a.step(2)
    a.checkpoint(tmp_path / "ck.bin")
    a.step(2)
    b = product.Simulation(cfg, types, rules)
    b.resume(tmp_path / "ck.bin")
    b.step(2)
    sa, sb = a.export_state(), b.export_state()
    assert sa[0].tobytes() == sb[0].tobytes()
    assert sa[1].tobytes() == sb[1].tobytes()
    ca, cb = a.counters(), b.counters()
    assert (ca.n_active_particles, ca.next_particle_id, ca.step) == (cb.n_active_particles, cb.next_particle_id,
                                                                      cb.step)
    a.close()
    b.close()
