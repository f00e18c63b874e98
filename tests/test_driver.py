"""The CMake build and sc_run, the spatial_cell_sim-style driver of the C ABI.

sc_run reads config.json and the type / rule tables like the reference's
main() (spatial_cell_sim/src/main.cu:142-338), generates its scene on the
device, steps and streams frames.dat (main.cu:95-126, storage.cuh:22-39).
On the GPU its frames.dat must hold exactly the frames the library gives
through the Python binding for the same config, tables and scene."""
import ctypes
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from spatial_cell_gb300 import abi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_tables(dirpath, types, rules):
    """The tables in the reference's JSON schemas (large-molecules.json,
    complexification.json)."""
    tj = [{"type": int(t), "radius": float(types[t]["radius"]), "hydrophobic": int(types[t]["hydrophobic"])}
          for t in range(len(types)) if types[t]["radius"] != 0]
    rj = []
    for r in rules:
        d = {"id": int(r["id"]), "group": int(r["group"]), "firstPartnerType": int(r["first_partner_type"]),
             "firstPartnerState": int(r["first_partner_state"]), "secondPartnerType": int(r["second_partner_type"]),
             "secondPartnerState": int(r["second_partner_state"]), "propagateState": bool(r["propagate_state"]),
             "setState": bool(r["set_state"]), "waitForState": bool(r["wait_for_state"]),
             "waitForAlignment": bool(r["wait_for_alignment"]), "onlyViaTransition": bool(r["only_via_transition"]),
             "transitionTo": int(r["transition_to"]), "polymerize": int(r["polymerize"]),
             "breakAfterTransition": bool(r["break_after_transition"]),
             "relativeOrientation": [float(x) for x in r["relative_orientation"]],
             "orientationAlignmentThreshold": float(r["orientation_alignment_threshold"]),
             "relativePosition": [float(x) for x in r["relative_position"]],
             "positionAlignmentThreshold": float(r["position_alignment_threshold"])}
        if r["use_probability"]:
            d["probability"] = float(r["probability"])
        rj.append(d)
    tp, rp = os.path.join(dirpath, "large-molecules.json"), os.path.join(dirpath, "complexification.json")
    with open(tp, "w") as f:
        json.dump(tj, f)
    with open(rp, "w") as f:
        json.dump(rj, f)
    return tp, rp


def write_config(path, cfg):
    keys = {"numParticles": cfg.num_particles, "numMetabolicParticles": cfg.num_metabolic_particles,
            "steps": cfg.steps, "simSize": cfg.sim_size, "maxInteractionDistance": cfg.max_interaction_distance,
            "maxDiffusionDistance": cfg.max_diffusion_distance, "gridCellSize": cfg.grid_cell_size,
            "movementNoiseScale": cfg.movement_noise_scale, "rotationNoiseScale": cfg.rotation_noise_scale,
            "metaboliteMovementNoiseScale": cfg.metabolite_movement_noise_scale,
            "velocityDecay": cfg.velocity_decay, "angularVelocityDecay": cfg.angular_velocity_decay,
            "noiseCoordinationSteps": cfg.noise_coordination_steps, "relaxationSteps": cfg.relaxation_steps,
            "metaboliteDiffusionSteps": cfg.metabolite_diffusion_steps,
            "persistEveryNthFrame": cfg.persist_every_nth_frame, "reportEveryNthFrame": cfg.report_every_nth_frame,
            "numMetabolites": cfg.num_metabolites, "periodic": cfg.periodic, "walls": cfg.walls,
            "pairClaim": cfg.pair_claim, "ruleProbabilities": cfg.rule_probabilities, "seed": int(cfg.seed)}
    with open(path, "w") as f:
        json.dump(keys, f)


@pytest.mark.skipif(shutil.which("cmake") is None, reason="cmake is not installed")
def test_cmake_build_exports_every_symbol(tmp_path):
    from spatial_cell_gb300 import native
    b = tmp_path / "build"
    subprocess.run(["cmake", "-S", ROOT, "-B", str(b), "-DCMAKE_BUILD_TYPE=Release"], check=True,
                   capture_output=True)
    subprocess.run(["cmake", "--build", str(b), "-j", "8"], check=True, capture_output=True)
    lib = ctypes.CDLL(str(b / "libspatialcell.so"))
    missing = [s for s in native.EXPORTED if not hasattr(lib, s)]
    assert not missing
    assert subprocess.run([str(b / "sc_run"), "--help"], capture_output=True).returncode == 0


def test_driver_is_built_in_tree(product):
    from spatial_cell_gb300 import build
    r = subprocess.run([build.DRIVER, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage: sc_run" in r.stderr


def test_config_json_round_trip(product, tmp_path):
    cfg = scenes.measured_config("plain_small", num_particles=1234, sim_size=77.0, walls=1, periodic=0)
    write_config(tmp_path / "config.json", cfg)
    back = product.load_config_json(str(tmp_path / "config.json"))
    for k, _ in abi.Config._fields_:
        if not k.startswith("_") and k not in ("graphs", "class_streams", "tiles", "pair_list_limit",
                                               "pool_per_item"):
            assert getattr(back, k) == getattr(cfg, k), k


@pytest.mark.gpu
def test_driver_frames_equal_the_library_frames(product, tmp_path):
    from spatial_cell_gb300 import build
    n, nm, steps, seed = 3000, 6000, 3, 77
    cfg = scenes.measured_config("plain_small", num_particles=n + 64, num_metabolic_particles=nm + 32,
                                 sim_size=float(200.0 * (n / 65536.0) ** (1.0 / 3.0)), steps=steps, seed=11)
    types, rules = scenes.baseline_types(), scenes.workload_rules()
    tp, rp = write_tables(str(tmp_path), types, rules)
    write_config(tmp_path / "config.json", cfg)
    frames = tmp_path / "frames.dat"
    mix = "0:0.4,1:0.4,2:0.1,3:0.1"
    r = subprocess.run([build.DRIVER, "--config", str(tmp_path / "config.json"), "--types", tp, "--rules", rp,
                        "--frames", str(frames), "--particles", str(n), "--metabolic", str(nm), "--mix", mix,
                        "--seed", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    # the same run through the Python binding
    t2 = product.load_types_json(tp)
    r2 = product.load_rules_json(rp)
    c2 = product.load_config_json(str(tmp_path / "config.json"))
    sim = product.Simulation(c2, t2, r2)
    sim.generate_uniform(n, nm, (0, 1, 2, 3), (0.4, 0.4, 0.1, 0.1), seed)
    sim.prepare()
    want = [struct_bytes(sim.reduce_frame())]
    for _ in range(steps):
        sim.step(1)
        want.append(struct_bytes(sim.reduce_frame()))
    sim.close()
    data = frames.read_bytes()
    head = np.frombuffer(data[:12], np.uint32)
    assert np.frombuffer(data[:4], np.float32)[0] == np.float32(cfg.sim_size)
    assert tuple(head[1:]) == (cfg.num_particles, cfg.num_metabolic_particles)
    off, got = 12, []
    for _ in range(steps + 1):
        k = 4 + cfg.num_particles * 36 + 4 + cfg.num_metabolic_particles * 44
        got.append(data[off:off + k])
        off += k
    assert off == len(data)
    for k, (g, w) in enumerate(zip(got, want)):
        assert g == w, f"frame {k} differs"


def struct_bytes(frame):
    rp, rm = frame
    return (np.uint32(len(rp)).tobytes() + rp.tobytes() + np.uint32(len(rm)).tobytes() + rm.tobytes())
