"""Synthetic workloads in the reference's state layout.

No dataset is involved anywhere in the reference: its scene is generated in
code (spatial_cell_sim/src/setup/setup.cuh:17-253).  These generators build
seeded states with the shapes, sizes and value ranges of the workloads this
project measures, in the reference's own ``Particle`` / ``MetabolicParticle``
layout, plus small scenes that exercise every branch of the step (chains,
rule bonds with transitions and polymerisation, test bonds, lipids).
"""
import numpy as np

from . import abi

LIPID, DUMMY, TYPE_A, TYPE_B = 0, 1, 2, 3
METABOLIC = abi.PARTICLE_TYPE_METABOLIC


def random_quaternions(rng, n):
    """Uniform random unit quaternions (Shoemake's method, as math.cuh:264-277)."""
    u, v, w = rng.random(n), rng.random(n), rng.random(n)
    su, su1 = np.sqrt(u), np.sqrt(1.0 - u)
    q = np.stack([su1 * np.sin(2 * np.pi * v), su1 * np.cos(2 * np.pi * v),
                  su * np.sin(2 * np.pi * w), su * np.cos(2 * np.pi * w)], axis=1)
    return q.astype(np.float32)


def blank_particles(n, dtype=abi.PARTICLE_DTYPE):
    """Particle(...) defaults of types.cuh:192-221 (active, identity rotations)."""
    p = np.zeros(n, dtype)
    p["flags"] = abi.PARTICLE_FLAG_ACTIVE
    p["last_state_change_step"] = -1
    p["rot"][:, 3] = 1.0
    p["angular_velocity"][:, 3] = 1.0
    p["angular_noise"][:, 3] = 1.0
    p["scheduled_polymerization"] = -1
    return p


def baseline_types():
    """Type table of the measured workloads: lipid r=1.0 (polar), dummy r=2.0,
    A and B r=2.5, metabolite carrier (type 1000) r=2.5; id-indexed."""
    t = np.zeros(METABOLIC + 1, abi.TYPE_INFO_DTYPE)
    t[LIPID] = (1.0, abi.POLAR)
    t[DUMMY] = (2.0, abi.HYDROPHYLIC)
    t[TYPE_A] = (2.5, abi.HYDROPHYLIC)
    t[TYPE_B] = (2.5, abi.HYDROPHYLIC)
    t[METABOLIC] = (2.5, abi.HYDROPHYLIC)
    return t


def rule(rid, first, second, group=None, first_state=-1, second_state=-1, set_state=1, wait_for_state=1,
         wait_for_alignment=1, only_via_transition=0, transition_to=-1, polymerize=-1, break_after=0,
         rel_ori=(0.0, 0.0, 0.0, 1.0), rel_pos=(0.0, 0.0, 0.0), ori_thr=0.8, pos_thr=0.8):
    """One complexification rule with the loader defaults of interactions.cuh:33-49."""
    r = np.zeros(1, abi.RULE_DTYPE)
    r["id"] = rid
    r["group"] = rid if group is None else group
    r["first_partner_type"] = first
    r["second_partner_type"] = second
    r["first_partner_state"] = first_state
    r["second_partner_state"] = second_state
    r["set_state"] = set_state
    r["wait_for_state"] = wait_for_state
    r["wait_for_alignment"] = wait_for_alignment
    r["only_via_transition"] = only_via_transition
    r["transition_to"] = transition_to
    r["polymerize"] = polymerize
    r["break_after_transition"] = break_after
    r["relative_orientation"] = rel_ori
    r["relative_position"] = rel_pos
    r["orientation_alignment_threshold"] = ori_thr
    r["position_alignment_threshold"] = pos_thr
    return r


def baseline_rules(probability=None):
    """A + B bind when their centres pass the interaction cube (alignment gates
    left open): one rule, group = id so each particle holds one such bond.
    With a probability the rule binds with it per step (an extension; the
    sim must be created with rule_probabilities = 1)."""
    r = rule(1001, TYPE_A, TYPE_B, rel_pos=(0.0, 5.0, 0.0), ori_thr=-2.0, pos_thr=-100.0)
    if probability is not None:
        r["use_probability"] = 1
        r["probability"] = probability
    return r


def uniform_particles(rng, n, box, types, fractions=((LIPID, 0.4), (DUMMY, 0.4), (TYPE_A, 0.1), (TYPE_B, 0.1))):
    p = blank_particles(n)
    counts = [int(n * f) for _, f in fractions]
    counts[1] += n - sum(counts)
    kinds = np.concatenate([np.full(c, t, np.int32) for (t, _), c in zip(fractions, counts)])
    kinds = rng.permutation(kinds)
    p["id"] = np.arange(n, dtype=np.int32)
    p["type"] = kinds
    p["radius"] = types["radius"][kinds]
    p["hydrophobic"] = types["hydrophobic"][kinds]
    p["pos"] = (rng.random((n, 3)) * box).astype(np.float32)
    p["rot"] = random_quaternions(rng, n)
    return p


def uniform_metabolic(rng, nm, box, types, species):
    m = blank_particles(nm, abi.METABOLIC_DTYPE)
    m["id"] = np.arange(nm, dtype=np.int32)
    m["type"] = METABOLIC
    m["radius"] = types["radius"][METABOLIC]
    m["hydrophobic"] = types["hydrophobic"][METABOLIC]
    m["pos"] = (rng.random((nm, 3)) * box).astype(np.float32)
    m["rot"] = random_quaternions(rng, nm)
    amounts = np.zeros((nm, abi.AOS_NUM_METABOLITES), np.float32)
    # species 0 seeded as in metabolite_setup.cuh:13-28, the others random
    amounts[:, 0] = np.where(m["pos"][:, 0] < box * 0.2, 100.0, 0.0)
    if species > 1:
        amounts[:, 1:species] = (rng.random((nm, species - 1)) * 10.0).astype(np.float32)
    m["metabolites"] = amounts
    return m


# Measured workloads.  Each is (particles, metabolic particles, box nm, cell nm, seed).
WORKLOADS = {
    "plain_small": dict(n=65536, nm=131072, box=200.0, seed=1),
    "plain_large": dict(n=2097152, nm=8388608, box=635.0, seed=2),
}


# The A + B binding probability per step of the measured workloads, and the
# extension switches they run with: complexify by deterministic pair claim,
# rule probabilities honoured.  (workload_config alone keeps the reference's
# complexify, for comparisons with the reference's own kernels.)
WORKLOAD_BIND_PROBABILITY = 0.1
WORKLOAD_EXTENSIONS = dict(pair_claim=1, rule_probabilities=1)


def workload_rules():
    """The measured workloads' rule table: A + B bind with probability 0.1 per step."""
    return baseline_rules(probability=WORKLOAD_BIND_PROBABILITY)


def measured_config(name, **overrides):
    """workload_config with the measured workloads' extension switches."""
    return workload_config(name, **{**WORKLOAD_EXTENSIONS, **overrides})


def workload_config(name, **overrides):
    w = WORKLOADS[name]
    kw = dict(num_particles=w["n"], num_metabolic_particles=w["nm"], sim_size=w["box"], grid_cell_size=6.0,
              max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8, seed=w["seed"],
              steps=200 if name == "plain_small" else 1000, periodic=1)
    kw.update(overrides)
    return abi.make_config(**kw)


def batch_specs(count, seed=3, n_lo=2048, n_hi=262144):
    """The replica cells of the batched workload without their states:
    (particles, metabolic, box nm, mix, seed) per replica, as batch_replicas
    draws them (states then come from sc_generate_batch on the device)."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        box = float(200.0 * (n / 65536.0) ** (1.0 / 3.0))
        mix = rng.dirichlet([2.0, 2.0, 1.0, 1.0])
        out.append((n, 2 * n, box, mix, seed * 1000 + r))
    return out


def batch_sim_args(specs, **overrides):
    """Config and replicas (abi.Replica) of a batch of replica specs."""
    cfg = measured_config("plain_small", num_particles=specs[0][0], num_metabolic_particles=specs[0][1],
                          sim_size=specs[0][2], seed=specs[0][4], **overrides)
    reps = [abi.Replica(n, nm, box, 0, sd) for n, nm, box, _, sd in specs]
    return cfg, reps


def batch_replicas(count, seed=3, n_lo=2048, n_hi=262144):
    """Replica cells of the batched workload: particle counts log-uniform in
    [n_lo, n_hi], twice as many metabolic items, each periodic cube scaled to
    the small workload's number density (65,536 particles in 200 nm), type mix
    (lipid, dummy, A, B) ~ Dirichlet(2, 2, 1, 1).  Returns a list of
    (config, types, rules, particles, metabolic) for seeds seed*1000 + r."""
    rng = np.random.default_rng(seed)
    types, rules = baseline_types(), workload_rules()
    out = []
    for r in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        nm = 2 * n
        box = float(200.0 * (n / 65536.0) ** (1.0 / 3.0))
        mix = rng.dirichlet([2.0, 2.0, 1.0, 1.0])
        cfg = measured_config("plain_small", num_particles=n, num_metabolic_particles=nm, sim_size=box,
                              seed=seed * 1000 + r)
        rr = np.random.default_rng(seed * 1000 + r)
        p = uniform_particles(rr, n, box, types, fractions=tuple(zip((LIPID, DUMMY, TYPE_A, TYPE_B), mix)))
        m = uniform_metabolic(rr, nm, box, types, cfg.num_metabolites)
        out.append((cfg, types, rules, p, m))
    return out


def vesicle_groups(box, shell_r=400.0, lipids=2_000_000, interior=6_000_000, complexes=50_000, complex_size=20,
                   spacing=3.0, leaflet_gap=4.0):
    """Scene groups of the crowded vesicle case: a lipid bilayer shell
    (two leaflets leaflet_gap apart, lipids uniform on each sphere and split
    by area, heads out on the outer leaflet and in on the inner one, as the
    reference's two fillParticlesSphere leaflets are oriented), interior
    particles dummy / A / B 70 / 15 / 15 uniform in the ball inside, and
    rigid-lattice complexes of dummies (complex_size sites on the cubic
    lattice of the given spacing, bonded along the growth tree with chain
    bonds) in the same ball."""
    c = (box / 2.0, box / 2.0, box / 2.0)
    ri = shell_r - leaflet_gap
    n_out = int(round(lipids * shell_r ** 2 / (shell_r ** 2 + ri ** 2)))
    inner = ri - 6.0
    return [
        abi.scene_group(abi.SCENE_SPHERE_SHELL, n_out, [LIPID], center=c, radius=shell_r),
        abi.scene_group(abi.SCENE_SPHERE_SHELL, lipids - n_out, [LIPID], center=c, radius=ri,
                        rot=(1.0, 0.0, 0.0, 0.0)),
        abi.scene_group(abi.SCENE_UNIFORM_BALL, interior, [DUMMY, TYPE_A, TYPE_B], [0.70, 0.15, 0.15], center=c,
                        radius=inner),
        abi.scene_group(abi.SCENE_COMPLEXES, complexes, [DUMMY], center=c, radius=inner - 2.0 * spacing,
                        unit=complex_size, spacing=spacing, link_type=abi.INTERACTION_TYPE_CHAIN),
    ]


def vesicle_workload(scale=1.0, **overrides):
    """The crowded vesicle stress case (900 nm box with reflecting walls, 2 M
    lipids on a 400 nm bilayer shell, 6 M interior particles, 50 k 20-particle complexes,
    32 M metabolic items, seed 5), every count scaled by `scale` and every
    length by its cube root, with the measured workloads' A + B binding
    (workload_rules: probability 0.1 per step, pair claim).  Returns
    (config, groups, metabolic count)."""
    s = scale ** (1.0 / 3.0)
    box = 900.0 * s
    groups = vesicle_groups(box, shell_r=400.0 * s, lipids=int(2_000_000 * scale), interior=int(6_000_000 * scale),
                            complexes=int(50_000 * scale))
    n = abi.scene_particles(groups)
    nm = int(32_000_000 * scale)
    kw = dict(num_particles=n, num_metabolic_particles=nm, sim_size=box, grid_cell_size=6.0,
              max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8, seed=5, steps=1000,
              periodic=0, walls=1, **WORKLOAD_EXTENSIONS)
    kw.update(overrides)
    return abi.make_config(**kw), groups, nm


def build_workload(name, **overrides):
    """Config, tables and initial state of a measured workload (the A + B rule
    at probability 0.1 per step, complexify by pair claim, periodic box)."""
    cfg = measured_config(name, **overrides)
    rng = np.random.default_rng(cfg.seed)
    types = baseline_types()
    rules = workload_rules()
    p = uniform_particles(rng, cfg.num_particles, cfg.sim_size, types)
    m = uniform_metabolic(rng, cfg.num_metabolic_particles, cfg.sim_size, types, cfg.num_metabolites)
    return cfg, types, rules, p, m


# ---------------------------------------------------------------------------
# Small scenes for differential testing: every branch of the step.
# ---------------------------------------------------------------------------
CHAIN_A, CHAIN_B, CHAIN_C = 40, 41, 42   # chain monomer types
CTRL, MONO = 50, 51                       # polymerising controller and its monomer
HALF_A, HALF_B = 60, 61                   # transition / break-after pair


def test_types():
    t = baseline_types()
    for ty, r, h in [(CHAIN_A, 0.75, 0), (CHAIN_B, 0.75, 0), (CHAIN_C, 0.8, 1), (CTRL, 2.0, 0), (MONO, 1.0, 0),
                     (HALF_A, 1.5, 1), (HALF_B, 1.7, 0)]:
        t[ty] = (r, h)
    return t


def test_rules():
    """Rules reaching every path of complexify / transitionInteractions /
    polymerize: alignment gates, states, groups, transitions that set state,
    break-after-transition, and a polymerising transition."""
    rs = [
        # A+B with real alignment gates
        rule(1001, TYPE_A, TYPE_B, rel_pos=(0.0, 4.0, 1.0), rel_ori=(0.0, 0.38268343, 0.0, 0.92387953),
             ori_thr=-0.3, pos_thr=-1.5, transition_to=1002),
        # formed only by transition; sets states, then breaks after aligning
        rule(1002, TYPE_A, TYPE_B, group=1001, first_state=1, second_state=2, only_via_transition=1,
             transition_to=1003, rel_pos=(0.0, 4.0, 1.0), ori_thr=-0.5, pos_thr=-2.0),
        rule(1003, TYPE_A, TYPE_B, group=1001, only_via_transition=1, break_after=1, rel_pos=(0.0, 4.0, 1.0)),
        # homotypic rule without group (may be granted twice)
        rule(1010, HALF_A, HALF_A, group=-1, rel_pos=(0.0, 3.0, 0.0), ori_thr=-1.0, pos_thr=-3.0),
        # HALF_A + HALF_B with state requirement
        rule(1011, HALF_A, HALF_B, first_state=0, second_state=-1, rel_pos=(3.2, 0.0, 0.0), ori_thr=-0.8,
             pos_thr=-3.0, transition_to=1012),
        rule(1012, HALF_A, HALF_B, group=1011, first_state=3, second_state=-1, only_via_transition=1,
             wait_for_alignment=0, rel_pos=(3.2, 0.0, 0.0)),
        # polymerisation: controller binds a monomer, a transition schedules a new monomer
        rule(1020, CTRL, MONO, group=1020, rel_pos=(0.0, 3.0, 0.0), ori_thr=-1.0, pos_thr=-4.0,
             transition_to=1021),
        rule(1021, CTRL, MONO, group=1020, first_state=1, only_via_transition=1, polymerize=1022,
             transition_to=1023, wait_for_alignment=0, rel_pos=(0.0, 3.0, 0.0)),
        rule(1022, CTRL, MONO, group=1020, only_via_transition=1, rel_pos=(0.0, 3.0, 0.0),
             rel_ori=(0.0, 0.0, 0.0, 1.0)),
        rule(1023, CTRL, MONO, group=1020, first_state=2, only_via_transition=1, wait_for_alignment=0,
             rel_pos=(0.0, 3.0, 0.0)),
    ]
    out = np.zeros(len(rs), abi.RULE_DTYPE)   # (np.concatenate would drop the padded layout)
    for i, r in enumerate(rs):
        out[i] = r[0]
    return out


def _link_serially(p, start, end, itype=abi.INTERACTION_TYPE_CHAIN):
    """linkParticlesSerially (setup/interaction_setup.cuh:13-42)."""
    for i in range(start + 1, end):
        a, b = p[i - 1], p[i]
        k = a["n_active_interactions"]
        a["interactions"][k] = (itype, abi.INTERACTION_GROUP_FORWARD, b["id"])
        a["n_active_interactions"] = k + 1
        k = b["n_active_interactions"]
        b["interactions"][k] = (itype, abi.INTERACTION_GROUP_BACKWARD, a["id"])
        b["n_active_interactions"] = k + 1


def test_scene(seed, n=1500, nm=3000, box=48.0, species=10, capacity_slack=64, periodic=0, walls=0):
    """A dense small box with uniform particles of all kinds, a few wrapped
    chains, pre-bonded rule pairs, a test bond, and metabolites.  Returns
    (config, types, rules, particles, metabolic, next_particle_id)."""
    rng = np.random.default_rng(seed)
    types = test_types()
    rules = test_rules()
    kinds = np.array([LIPID, DUMMY, TYPE_A, TYPE_B, HALF_A, HALF_B, CTRL, MONO, CHAIN_C])
    weights = np.array([0.35, 0.2, 0.1, 0.1, 0.06, 0.06, 0.04, 0.05, 0.04])
    p = blank_particles(n)
    ty = rng.choice(kinds, size=n, p=weights / weights.sum()).astype(np.int32)
    p["id"] = np.arange(n, dtype=np.int32)
    p["type"] = ty
    p["radius"] = types["radius"][ty]
    p["hydrophobic"] = types["hydrophobic"][ty]
    p["pos"] = (rng.random((n, 3)) * box).astype(np.float32)
    p["rot"] = random_quaternions(rng, n)
    p["velocity"] = (rng.normal(size=(n, 3)) * 0.2).astype(np.float32)
    p["angular_velocity"] = random_quaternions(rng, n)
    p["angular_velocity"][:, 3] += 8.0           # near-identity angular velocities
    p["angular_velocity"] /= np.linalg.norm(p["angular_velocity"], axis=1, keepdims=True)
    p["state"] = rng.choice([0, 0, 0, 1, 2, 3], size=n)
    # chains: consecutive ids placed along a straight segment
    c0, r0, t0 = int(0.07 * n), int(0.6 * n), int(0.8 * n)   # where chains, bonded pairs, the test bond go
    assert n >= 300, "the differential scene needs at least 300 particles"
    for c in range(6):
        length = 8
        start = c0 + c * 20
        q = rng.random(3) * (box - 12) + 6
        step = rng.normal(size=3)
        step /= np.linalg.norm(step)
        for i in range(start, start + length):
            p[i]["type"] = CHAIN_A if (i - start) % 2 == 0 else CHAIN_B
            p[i]["radius"] = types["radius"][p[i]["type"]]
            p[i]["hydrophobic"] = 0
            p[i]["pos"] = (q + step * 1.5 * (i - start)).astype(np.float32)
        _link_serially(p, start, start + length)
    # rule bonds already formed (both directions), including one that transitions
    for k in range(10):
        a, b = r0 + 2 * k, r0 + 1 + 2 * k
        p[a]["type"], p[b]["type"] = (TYPE_A, TYPE_B) if k % 2 == 0 else (CTRL, MONO)
        for i in (a, b):
            p[i]["radius"] = types["radius"][p[i]["type"]]
            p[i]["hydrophobic"] = 0
        p[b]["pos"] = (p[a]["pos"] + rng.normal(size=3).astype(np.float32) * 1.5).clip(0, box)
        rid = 1001 if k % 2 == 0 else 1020
        for i, j in ((a, b), (b, a)):
            kk = p[i]["n_active_interactions"]
            p[i]["interactions"][kk] = (rid, 1001 if rid == 1001 else 1020, p[j]["id"])
            p[i]["n_active_interactions"] = kk + 1
        if k % 2 == 1:
            p[a]["state"] = 1
    # a test bond (interaction type 0) between two close particles
    p[t0]["pos"] = p[t0 + 1]["pos"] + np.float32(2.0)
    for i, j in ((t0, t0 + 1), (t0 + 1, t0)):
        kk = p[i]["n_active_interactions"]
        p[i]["interactions"][kk] = (0, -1, p[j]["id"])
        p[i]["n_active_interactions"] = kk + 1
    p["pos"] = p["pos"].clip(0, box)
    m = uniform_metabolic(rng, nm, box, types, species)
    m["velocity"] = (rng.normal(size=(nm, 3)) * 0.3).astype(np.float32)
    cfg = abi.make_config(num_particles=n + capacity_slack, num_metabolic_particles=nm + 16, sim_size=box,
                          grid_cell_size=6.0, max_interaction_distance=5.5, max_diffusion_distance=6.0,
                          num_metabolites=species, seed=1000 + seed, noise_coordination_steps=4,
                          relaxation_steps=6, metabolite_diffusion_steps=3, steps=10, periodic=periodic,
                          walls=walls)
    return cfg, types, rules, p, m, n


def polymer_scene(seed, pairs, scheduled_monomers=0, shared=0, capacity_slack=None, box=None):
    """Controllers, each bonded (rule 1022, group 1020, both directions) to a
    monomer 1.5-3 nm away and scheduled to polymerise by rule 1022, which
    creates a new monomer.  `scheduled_monomers` monomers are scheduled too
    (their previous monomer -- the controller -- is then itself scheduled);
    `shared` monomers are bonded to a second controller as well (two
    scheduled items share a previous monomer).  Capacity: the particles plus
    `capacity_slack` (default: room for every new monomer).  Returns
    (config, types, rules, particles, metabolic, next_particle_id)."""
    rng = np.random.default_rng(seed)
    types, rules = test_types(), test_rules()
    n = 2 * pairs
    box = float(box or 3.0 * (n ** (1.0 / 3.0)) + 12.0)
    p = blank_particles(n)
    p["id"] = np.arange(n, dtype=np.int32)
    ctrl, mono = np.arange(0, n, 2), np.arange(1, n, 2)
    p["type"][ctrl], p["type"][mono] = CTRL, MONO
    p["radius"] = types["radius"][p["type"]]
    p["rot"] = random_quaternions(rng, n)
    p["pos"][ctrl] = (rng.random((pairs, 3)) * (box - 8.0) + 4.0).astype(np.float32)
    off = rng.normal(size=(pairs, 3))
    off *= (rng.uniform(1.5, 3.0, pairs) / np.linalg.norm(off, axis=1))[:, None]
    p["pos"][mono] = (p["pos"][ctrl] + off).astype(np.float32)
    for c, m in zip(ctrl, mono):
        p[c]["interactions"][0] = (1022, 1020, p[m]["id"])
        p[m]["interactions"][0] = (1022, 1020, p[c]["id"])
    p["n_active_interactions"] = 1
    p["scheduled_polymerization"] = -1
    p["scheduled_polymerization"][ctrl] = 1022
    if scheduled_monomers:
        p["scheduled_polymerization"][rng.choice(mono, scheduled_monomers, replace=False)] = 1022
    if shared:
        # controller k + 1 also bonds controller k's monomer, placed between them
        for k in rng.choice(pairs - 1, shared, replace=False):
            c2, m = ctrl[k + 1], mono[k]
            p[c2]["pos"] = p[m]["pos"] + np.float32(1.0)
            p[c2]["interactions"][0] = (1022, 1020, p[m]["id"])
            j = p[m]["n_active_interactions"]
            if j < abi.MAX_ACTIVE_INTERACTIONS:
                p[m]["interactions"][j] = (1022, 1020, p[c2]["id"])
                p[m]["n_active_interactions"] = j + 1
    p["pos"] = p["pos"].clip(0, box)
    slack = pairs + scheduled_monomers + 16 if capacity_slack is None else capacity_slack
    m = uniform_metabolic(rng, 64, box, types, 8)
    cfg = abi.make_config(num_particles=n + slack, num_metabolic_particles=64, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8,
                          seed=2000 + seed, noise_coordination_steps=4, relaxation_steps=6,
                          metabolite_diffusion_steps=3, steps=10)
    return cfg, types, rules, p, m, n


def propagation_scene(seed, chains=300, length=6, n_free=600):
    """Chains of particles bonded to their neighbours by rule bonds -- rule
    1001 (which propagates state) on even chains, rule 1010 (which does not)
    on odd ones -- with random states and last state-change steps, among free
    particles, in a box the chains fill; config with propagate_state on.
    Returns (config, types, rules, particles, metabolic, next_particle_id)."""
    rng = np.random.default_rng(seed)
    types, rules = test_types(), test_rules()
    rules["propagate_state"] = 0
    rules["propagate_state"][rules["id"] == 1001] = 1
    n = chains * length + n_free
    box = float(2.2 * n ** (1.0 / 3.0) + 10.0)
    p = blank_particles(n)
    p["id"] = np.arange(n, dtype=np.int32)
    p["type"] = rng.choice([TYPE_A, TYPE_B, DUMMY], size=n)
    p["radius"] = types["radius"][p["type"]]
    p["rot"] = random_quaternions(rng, n)
    p["pos"] = (rng.random((n, 3)) * (box - 10.0) + 5.0).astype(np.float32)
    for c in range(chains):
        s0 = c * length
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        for k in range(length):
            p[s0 + k]["pos"] = (p[s0]["pos"] + d * 1.8 * k).astype(np.float32)
        _link_serially(p, s0, s0 + length, itype=1001 if c % 2 == 0 else 1010)
    p["pos"] = p["pos"].clip(0, box)
    p["state"] = rng.integers(0, 4, n)
    p["last_state_change_step"] = rng.integers(-1, 60, n)
    m = uniform_metabolic(rng, 256, box, types, 8)
    cfg = abi.make_config(num_particles=n + 32, num_metabolic_particles=256 + 16, sim_size=box, grid_cell_size=6.0,
                          max_interaction_distance=5.5, max_diffusion_distance=6.0, num_metabolites=8,
                          seed=3000 + seed, noise_coordination_steps=4, relaxation_steps=6,
                          metabolite_diffusion_steps=3, steps=10, propagate_state=1)
    return cfg, types, rules, p, m, n


def batch_of(replica_states):
    """The batched-sim form of replica cells (as batch_replicas gives them):
    the shared config (replica 0's; the others differ only in capacities,
    box and seed) and one abi.Replica per cell."""
    cfg0 = replica_states[0][0]
    reps = [abi.Replica(c.num_particles, c.num_metabolic_particles, c.sim_size, 0, c.seed)
            for c, *_ in replica_states]
    return cfg0, reps
