"""The C ABI on the host (no GPU needed): the library loads and exports every
function include/spatialcell.h declares, the byte layouts match the
reference's structs, the setup-surface loaders follow jsoncpp's rules, the
frames.dat writer produces FileStorage's format, and invalid arguments are
rejected before any CUDA call."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

from spatial_cell_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "spatialcell.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sc_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(product):
    L = product.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), f"{n} is declared in spatialcell.h but not exported"
    assert set(names) == set(product.EXPORTED)


def test_layouts_are_the_reference_structs():
    assert abi.PARTICLE_DTYPE.itemsize == 256 and abi.METABOLIC_DTYPE.itemsize == 304
    assert abi.REDUCED_DTYPE.itemsize == 36 and abi.REDUCED_METABOLIC_DTYPE.itemsize == 44
    assert abi.RULE_DTYPE.itemsize == 96 and abi.TYPE_INFO_DTYPE.itemsize == 8
    f = abi.PARTICLE_DTYPE.fields
    assert (f["pos"][1], f["rot"][1], f["velocity"][1], f["angular_velocity"][1], f["interactions"][1],
            f["debug_vector"][1]) == (28, 48, 64, 96, 132, 240)
    assert abi.RULE_DTYPE.fields["relative_position"][1] == 68


def test_config_defaults_match_reference_config_json(product):
    c = abi.Config()
    product.lib().sc_config_defaults(ctypes.byref(c))
    ref = abi.make_config()
    for k, _ in abi.Config._fields_:
        if k.startswith("_"):
            continue
        assert getattr(c, k) == getattr(ref, k), k


def test_grid_derivation(product):
    # config.cuh:65-74: cells per axis = next power of two >= ceil(size / cell), at least 2
    for size, cell, want in [(400, 10, (64, 6)), (200, 6, (64, 6)), (635, 6, (128, 7)), (900, 6, (256, 8)),
                             (10, 10, (2, 1)), (1, 10, (2, 1)), (12, 6, (2, 1)), (12.5, 6, (4, 2))]:
        cfg = abi.make_config(sim_size=size, grid_cell_size=cell)
        assert product.grid(cfg) == want, (size, cell)
        assert abi.grid_dims(cfg)[:2] == want


def test_rule_loader_jsoncpp_rules(product, tmp_path):
    p = tmp_path / "rules.json"
    p.write_text("""[
      {"id": 1001, "firstPartnerType": 3, "secondPartnerType": 4,
       "relativeOrientation": [0, 0, 0, 1], "relativePosition": [1.5, -2, 0.1]},
      {"id": 1002, "group": 7, "firstPartnerType": 3, "secondPartnerType": 5, "polymerize": null,
       "transitionTo": 1001.9, "setState": 0, "waitForState": false, "firstPartnerState": 2,
       "orientationAlignmentThreshold": 0.5, "positionAlignmentThreshold": 1,
       "relativeOrientation": [0.1, 0.2, 0.3, 0.4], "relativePosition": [0, 0, 0]}
    ]""")
    r = product.load_rules_json(str(p))
    a, b = r[0], r[1]
    # defaults of interactions.cuh:33-49
    assert (a["group"], a["first_partner_state"], a["second_partner_state"], a["set_state"], a["wait_for_state"],
            a["wait_for_alignment"], a["only_via_transition"], a["transition_to"], a["polymerize"],
            a["break_after_transition"], a["propagate_state"]) == (-1, -1, -1, 1, 1, 1, 0, -1, -1, 0, 0)
    assert a["orientation_alignment_threshold"] == np.float32(0.8)
    assert a["position_alignment_threshold"] == np.float32(0.8)
    assert list(a["relative_position"]) == [np.float32(1.5), np.float32(-2.0), np.float32(0.1)]
    # explicit null -> 0, real literal read as int -> truncated, 0 / false -> false
    assert b["polymerize"] == 0 and b["transition_to"] == 1001
    assert b["set_state"] == 0 and b["wait_for_state"] == 0 and b["first_partner_state"] == 2
    assert b["position_alignment_threshold"] == 1.0


def test_type_loader(product, tmp_path):
    p = tmp_path / "types.json"
    p.write_text('[{"type": 0, "radius": 1.0, "hydrophobic": 2}, {"type": 5, "radius": 2.25},'
                 ' {"type": 5, "radius": 9.0}]')
    t = product.load_types_json(str(p))
    assert len(t) == 6
    assert tuple(t[0]) == (1.0, 2) and tuple(t[5]) == (2.25, 0) and tuple(t[3]) == (0.0, 0)


def test_loader_errors(product, tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('[{"type": 0, "radius": }]')
    with pytest.raises(product.ScError):
        product.load_types_json(str(bad))
    with pytest.raises(product.ScError):
        product.load_rules_json(str(tmp_path / "missing.json"))


def test_frames_writer_format(product, tmp_path):
    """storage.cuh:22-39: f32 simSize, u32 N, u32 Nm, then per frame u32 N,
    N x 36 bytes, u32 Nm, Nm x 44 bytes."""
    libc = ctypes.CDLL(None)
    libc.fopen.restype = ctypes.c_void_p
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [ctypes.c_void_p]
    cfg = abi.make_config(num_particles=3, num_metabolic_particles=2, sim_size=123.5)
    rp = np.zeros(3, abi.REDUCED_DTYPE)
    rp["id"] = [7, 8, 9]
    rm = np.zeros(2, abi.REDUCED_METABOLIC_DTYPE)
    rm["metabolites"][:, 0] = 0x3c00
    path = str(tmp_path / "frames.dat")
    f = libc.fopen(path.encode(), b"wb")
    L = product.lib()
    assert L.sc_frames_write_header(f, ctypes.byref(cfg)) == 0
    assert L.sc_frames_write_frame(f, ctypes.byref(cfg), abi.ptr(rp), abi.ptr(rm)) == 0
    libc.fclose(f)
    data = open(path, "rb").read()
    assert struct.unpack("<fII", data[:12]) == (123.5, 3, 2)
    assert struct.unpack("<I", data[12:16])[0] == 3
    assert data[16:16 + 108] == rp.tobytes()
    assert struct.unpack("<I", data[124:128])[0] == 2
    assert data[128:] == rm.tobytes()


def test_invalid_arguments_rejected_before_cuda(product):
    L = product.lib()
    h = ctypes.c_void_p()
    types = np.zeros(4, abi.TYPE_INFO_DTYPE)
    for kw in (dict(num_metabolites=0), dict(num_metabolites=11), dict(num_particles=-1),
               dict(grid_cell_size=0.0), dict(sim_size=1e6, grid_cell_size=0.5), dict(relaxation_steps=-1),
               dict(periodic=1, sim_size=12.0, grid_cell_size=6.0)):
        cfg = abi.make_config(**kw)
        rc = L.sc_create(ctypes.byref(cfg), abi.ptr(types), 4, None, 0, ctypes.byref(h))
        assert rc == -1, kw
        assert L.sc_last_error(None)
    assert L.sc_step(None, 1) == -1
    assert L.sc_load_state(None, None, 0, None, 0, 0, 0) == -1
