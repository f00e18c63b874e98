// sc_gen.h -- the uniform scene generator's records (host + device).
//
// A replacement for the reference's host-side scene setup of uniformly
// placed particles (setup/particle_setup.cuh, uniform placement with
// std::mt19937) that runs on the device: every record is a pure function of
// (seed, index), drawn from the step's counter-based Philox on two streams
// of its own, so the scene needs no host generation and no host-to-device
// copy.  The records are the reference's Particle / MetabolicParticle
// defaults (types.cuh:192-242: active, identity angular velocity and noise,
// no interactions, last state change and scheduled polymerisation -1) with:
//   particles   type chosen by one uniform draw against the cumulative mix,
//               position uniform in the box, orientation a uniform random
//               rotation (math.cuh:264-277 from three draws);
//   metabolic   type 1000, position and orientation the same way, species 0
//               at 100 in the slab x < 0.2 * box and 0 elsewhere
//               (metabolite_setup.cuh:13-28), species 1 .. S-1 uniform in
//               [0, 10).
// The CPU oracle builds the same records from this header; the device path
// writes them and loads them through the same unpacking as sc_load_state.
#pragma once

#include <string.h>

#include "scmath.h"
#include "spatialcell.h"

#define SC_GEN_STREAM_P 8u
#define SC_GEN_STREAM_M 9u

// Mix of up to four particle kinds: cumulative fractions, kinds, and each
// kind's radius / hydrophobicity from the type table.
typedef struct sc_gen_mix {
    float cum[4];
    int32_t kind[4];
    float radius[4];
    int8_t hydrophobic[4];
    int32_t nkinds;
} sc_gen_mix;

// The mix of `nkinds` kinds with relative weights `fractions` (normalised to
// cumulative fractions), radii from the type table.  0 on success, -1 for a
// kind outside the table, a negative weight or no kind.
SC_HD int sc_gen_make_mix(sc_gen_mix *mix, const int32_t *kinds, const float *fractions, int32_t nkinds,
                          const sc_type_info *types, int32_t ntypes) {
    memset(mix, 0, sizeof *mix);
    if (nkinds < 1 || nkinds > 4) return -1;
    mix->nkinds = nkinds;
    float acc = 0.0f;
    for (int k = 0; k < nkinds; k++) {
        if (kinds[k] < 0 || kinds[k] >= ntypes || !(fractions[k] >= 0.0f)) return -1;
        acc += fractions[k];
        mix->cum[k] = acc;
        mix->kind[k] = kinds[k];
        mix->radius[k] = types[kinds[k]].radius;
        mix->hydrophobic[k] = types[kinds[k]].hydrophobic;
    }
    for (int k = 0; k < nkinds; k++) mix->cum[k] = acc > 0.0f ? mix->cum[k] / acc : mix->cum[k];
    return 0;
}

SC_HD void sc_gen_blank(sc_particle *r) {
    memset(r, 0, sizeof *r);
    r->flags = SC_PARTICLE_FLAG_ACTIVE;
    r->last_state_change_step = -1;
    r->rot[3] = 1.0f;
    r->angular_velocity[3] = 1.0f;
    r->angular_noise[3] = 1.0f;
    r->scheduled_polymerization = -1;
}

SC_HD void sc_gen_particle(sc_particle *r, int32_t i, float box, const sc_gen_mix *mix, uint64_t seed) {
    sc_gen_blank(r);
    const uint32_t id = (uint32_t)i;
    const float u = sc_uniform(seed, SC_GEN_STREAM_P, id, 0, 0);
    int k = 0;
    while (k < mix->nkinds - 1 && !(u < mix->cum[k])) k++;
    r->id = i;
    r->type = mix->kind[k];
    r->radius = mix->radius[k];
    r->hydrophobic = mix->hydrophobic[k];
    for (int a = 0; a < 3; a++) r->pos[a] = sc_uniform(seed, SC_GEN_STREAM_P, id, 0, 1u + (uint32_t)a) * box;
    sc_f4 q = sc_random_rotation(sc_uniform(seed, SC_GEN_STREAM_P, id, 0, 4), sc_uniform(seed, SC_GEN_STREAM_P, id, 0, 5),
                                 sc_uniform(seed, SC_GEN_STREAM_P, id, 0, 6));
    r->rot[0] = q.x;
    r->rot[1] = q.y;
    r->rot[2] = q.z;
    r->rot[3] = q.w;
}

SC_HD void sc_gen_metabolic(sc_metabolic_particle *r, int32_t j, float box, int species, float radius,
                            int8_t hydrophobic, uint64_t seed) {
    memset(r->metabolites, 0, sizeof r->metabolites);
    memset(r->_pad, 0, sizeof r->_pad);
    sc_gen_blank(&r->p);
    const uint32_t id = (uint32_t)j;
    r->p.id = j;
    r->p.type = SC_PARTICLE_TYPE_METABOLIC;
    r->p.radius = radius;
    r->p.hydrophobic = hydrophobic;
    for (int a = 0; a < 3; a++) r->p.pos[a] = sc_uniform(seed, SC_GEN_STREAM_M, id, 0, (uint32_t)a) * box;
    sc_f4 q = sc_random_rotation(sc_uniform(seed, SC_GEN_STREAM_M, id, 0, 3), sc_uniform(seed, SC_GEN_STREAM_M, id, 0, 4),
                                 sc_uniform(seed, SC_GEN_STREAM_M, id, 0, 5));
    r->p.rot[0] = q.x;
    r->p.rot[1] = q.y;
    r->p.rot[2] = q.z;
    r->p.rot[3] = q.w;
    r->metabolites[0] = r->p.pos[0] < box * 0.2f ? 100.0f : 0.0f;
    for (int s = 1; s < species && s < SC_AOS_NUM_METABOLITES; s++)
        r->metabolites[s] = sc_uniform(seed, SC_GEN_STREAM_M, id, 0, 6u + (uint32_t)s) * 10.0f;
}
