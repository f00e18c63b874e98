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

// ---- structured scenes (sc_generate_scene) -----------------------------------
// Group g draws on stream SC_GEN_STREAM_SCENE + g, keyed by its unit index
// (a particle, or a whole complex / chain); the layout of the draws of a
// unit is fixed per kind, so every record is a function of (seed, group,
// unit) and the oracle builds the same records from this header.
#define SC_GEN_STREAM_SCENE 16u
#define SC_GEN_BALL_TRIES 32
#define SC_GEN_SITE_TRIES 16
#define SC_GEN_D_ROT 100u       // chains / complexes: first draw of the rotations
#define SC_GEN_D_SITES 1024u    // complexes: first draw of the lattice growth
#define SC_GEN_D_KINDS 8192u    // complexes: first draw of the member kinds

// A validated scene group with what its kernel needs from the type table.
typedef struct sc_gen_group {
    int32_t kind, count, unit, first;  // first: index of the group's first particle
    sc_gen_mix mix;
    float prevRadius[4];               // chains: radius of type id (kind - 1)
    float center[3], radius, spacing;
    float rot[4];
    int32_t link;
    uint32_t stream;
} sc_gen_group;

// Particles of a group and its work units.
SC_HD int64_t sc_gen_group_particles(int32_t kind, int32_t count, int32_t unit) {
    return (kind == SC_SCENE_COMPLEXES || kind == SC_SCENE_WRAPPED_CHAINS) ? (int64_t)count * unit : (int64_t)count;
}

SC_HD float sc_gen_u(const sc_gen_group *G, uint64_t seed, int32_t u, uint32_t d) {
    return sc_uniform(seed, G->stream, (uint32_t)u, 0, d);
}

SC_HD int sc_gen_pick(const sc_gen_mix *mix, float u) {
    int k = 0;
    while (k < mix->nkinds - 1 && !(u < mix->cum[k])) k++;
    return k;
}

// Record of particle `id` of kind index k at pos (clamped into the box) with
// orientation q, as the reference's helpers construct it.
SC_HD void sc_gen_put(sc_particle *r, int32_t id, const sc_gen_mix *mix, int k, sc_f3 pos, sc_f4 q, float box) {
    sc_gen_blank(r);
    r->id = id;
    r->type = mix->kind[k];
    r->radius = mix->radius[k];
    r->hydrophobic = mix->hydrophobic[k];
    r->pos[0] = fminf(fmaxf(pos.x, 0.0f), box);
    r->pos[1] = fminf(fmaxf(pos.y, 0.0f), box);
    r->pos[2] = fminf(fmaxf(pos.z, 0.0f), box);
    r->rot[0] = q.x;
    r->rot[1] = q.y;
    r->rot[2] = q.z;
    r->rot[3] = q.w;
}

// A point uniform in the unit ball from draws d0, d0 + 1, ... (rejection from
// the cube, at most SC_GEN_BALL_TRIES tries; the centre if all miss).
SC_HD sc_f3 sc_gen_ball(const sc_gen_group *G, uint64_t seed, int32_t u, uint32_t d0) {
    for (uint32_t t = 0; t < SC_GEN_BALL_TRIES; t++) {
        sc_f3 p = sc_make_f3(2.0f * sc_gen_u(G, seed, u, d0 + 3 * t) - 1.0f,
                             2.0f * sc_gen_u(G, seed, u, d0 + 3 * t + 1) - 1.0f,
                             2.0f * sc_gen_u(G, seed, u, d0 + 3 * t + 2) - 1.0f);
        if (dot(p, p) <= 1.0f) return p;
    }
    return sc_zero3();
}

SC_HD void sc_gen_link(sc_particle *a, sc_particle *b, int32_t type) {
    if (a->n_active_interactions < SC_MAX_ACTIVE_INTERACTIONS) {
        sc_interaction *x = &a->interactions[a->n_active_interactions++];
        x->type = type;
        x->group = SC_INTERACTION_GROUP_FORWARD;
        x->partner_id = b->id;
    }
    if (b->n_active_interactions < SC_MAX_ACTIVE_INTERACTIONS) {
        sc_interaction *x = &b->interactions[b->n_active_interactions++];
        x->type = type;
        x->group = SC_INTERACTION_GROUP_BACKWARD;
        x->partner_id = a->id;
    }
}

// A shell point's record: pos = centre + point * radius, oriented
// quaternionFromTo(up, normalize(pos - centre)) * rot (particle_setup.cuh:207-232).
SC_HD void sc_gen_shell_put(sc_particle *r, const sc_gen_group *G, int32_t id, int k, sc_f3 point, float box) {
    const sc_f3 c = sc_make_f3(G->center[0], G->center[1], G->center[2]);
    const sc_f3 pos = c + point * G->radius;
    const sc_f3 dir = normalize(pos - c);
    const sc_f4 q = sc_qmul(sc_quat_from_to(sc_up(), dir), sc_make_f4(G->rot[0], G->rot[1], G->rot[2], G->rot[3]));
    sc_gen_put(r, id, &G->mix, k, pos, q, box);
}

// Point i (1-based) of the n-point Fibonacci spiral (particle_setup.cuh:
// 176-195): latitude asin(-1 + 2i/(n+1)), longitude i golden angles; the
// longitude is reduced modulo 2 pi in double precision before the float
// sine / cosine.
SC_HD sc_f3 sc_gen_fibonacci(int32_t i, int32_t n) {
    const double gr = (2.2360679774997898 + 1.0) / 2.0;
    const double ga = (2.0 - gr) * (2.0 * 3.14159265358979323846);
    const double t = -1.0 + 2.0 * (double)i / (double)(n + 1);
    const double lon = ga * (double)i;
    const double twoPi = 2.0 * 3.14159265358979323846;
    const double lr = lon - floor(lon / twoPi) * twoPi;
    const float clat = (float)sqrt(1.0 - t * t);
    const float lf = (float)lr;
    return sc_make_f3(sc_cosf(lf) * clat, sc_sinf(lf) * clat, (float)t);
}

// Writes work unit u of group G: one record (out[0]) for the particle
// kinds, G->unit records for a complex or a chain.
SC_HD void sc_gen_unit(sc_particle *out, const sc_gen_group *G, int32_t u, float box, uint64_t seed) {
    const sc_f3 c = sc_make_f3(G->center[0], G->center[1], G->center[2]);
    switch (G->kind) {
        case SC_SCENE_UNIFORM_BOX: {
            const int k = sc_gen_pick(&G->mix, sc_gen_u(G, seed, u, 0));
            const sc_f3 p = sc_make_f3(sc_gen_u(G, seed, u, 1) * box, sc_gen_u(G, seed, u, 2) * box,
                                       sc_gen_u(G, seed, u, 3) * box);
            const sc_f4 q = sc_random_rotation(sc_gen_u(G, seed, u, 4), sc_gen_u(G, seed, u, 5), sc_gen_u(G, seed, u, 6));
            sc_gen_put(out, G->first + u, &G->mix, k, p, q, box);
            break;
        }
        case SC_SCENE_UNIFORM_BALL: {
            const int k = sc_gen_pick(&G->mix, sc_gen_u(G, seed, u, 0));
            const sc_f4 q = sc_random_rotation(sc_gen_u(G, seed, u, 1), sc_gen_u(G, seed, u, 2), sc_gen_u(G, seed, u, 3));
            const sc_f3 p = c + sc_gen_ball(G, seed, u, 4) * G->radius;
            sc_gen_put(out, G->first + u, &G->mix, k, p, q, box);
            break;
        }
        case SC_SCENE_SPHERE_SHELL: {
            const int k = sc_gen_pick(&G->mix, sc_gen_u(G, seed, u, 0));
            const float z = 2.0f * sc_gen_u(G, seed, u, 1) - 1.0f;
            const float phi = SC_2PI_F * sc_gen_u(G, seed, u, 2);
            const float s = sqrtf(fmaxf(0.0f, 1.0f - z * z));
            sc_gen_shell_put(out, G, G->first + u, k, sc_make_f3(s * sc_cosf(phi), s * sc_sinf(phi), z), box);
            break;
        }
        case SC_SCENE_FIBONACCI_SHELL: {
            const int k = sc_gen_pick(&G->mix, sc_gen_u(G, seed, u, 0));
            sc_gen_shell_put(out, G, G->first + u, k, sc_gen_fibonacci(u + 1, G->count), box);
            break;
        }
        case SC_SCENE_COMPLEXES: {
            const int n = G->unit;
            int sx[SC_SCENE_MAX_UNIT], sy[SC_SCENE_MAX_UNIT], sz[SC_SCENE_MAX_UNIT], par[SC_SCENE_MAX_UNIT];
            sx[0] = sy[0] = sz[0] = 0;
            par[0] = -1;
            for (int s = 1; s < n; s++) {
                int found = 0;
                for (int t = 0; t < SC_GEN_SITE_TRIES + 1 && !found; t++) {
                    for (int scan = 0; scan < (t < SC_GEN_SITE_TRIES ? 1 : s * 6) && !found; scan++) {
                        int p, dir;
                        if (t < SC_GEN_SITE_TRIES) {  // a random neighbour of a random earlier site
                            const uint32_t d = SC_GEN_D_SITES + 2u * (uint32_t)(s * SC_GEN_SITE_TRIES + t);
                            p = (int)(sc_gen_u(G, seed, u, d) * (float)s);
                            dir = (int)(sc_gen_u(G, seed, u, d + 1) * 6.0f);
                            p = p < s ? p : s - 1;
                            dir = dir < 6 ? dir : 5;
                        } else {  // all tries taken: the first free neighbour in order
                            p = scan / 6;
                            dir = scan % 6;
                        }
                        const int ax = dir >> 1, sg = (dir & 1) ? -1 : 1;
                        const int x = sx[p] + (ax == 0 ? sg : 0), y = sy[p] + (ax == 1 ? sg : 0),
                                  z = sz[p] + (ax == 2 ? sg : 0);
                        int taken = 0;
                        for (int q = 0; q < s; q++) taken |= (sx[q] == x && sy[q] == y && sz[q] == z);
                        if (!taken) {
                            sx[s] = x;
                            sy[s] = y;
                            sz[s] = z;
                            par[s] = p;
                            found = 1;
                        }
                    }
                }
            }
            const sc_f4 q = sc_random_rotation(sc_gen_u(G, seed, u, SC_GEN_D_ROT), sc_gen_u(G, seed, u, SC_GEN_D_ROT + 1),
                                               sc_gen_u(G, seed, u, SC_GEN_D_ROT + 2));
            const sc_f3 cc = c + sc_gen_ball(G, seed, u, 0) * G->radius;
            const int32_t id0 = G->first + u * n;
            for (int s = 0; s < n; s++) {
                const int k = sc_gen_pick(&G->mix, sc_gen_u(G, seed, u, SC_GEN_D_KINDS + (uint32_t)s));
                const sc_f3 off = sc_make_f3((float)sx[s] * G->spacing, (float)sy[s] * G->spacing, (float)sz[s] * G->spacing);
                sc_gen_put(&out[s], id0 + s, &G->mix, k, cc + sc_rotate(off, q), q, box);
            }
            for (int s = 1; s < n; s++) sc_gen_link(&out[par[s]], &out[s], G->link);
            break;
        }
        case SC_SCENE_WRAPPED_CHAINS: {
            // particle_setup.cuh:78-117 and interaction_setup.cuh:13-43
            const int n = G->unit;
            sc_f3 pos = c + sc_gen_ball(G, seed, u, 0) * G->radius;
            sc_f4 rot = sc_random_rotation(sc_gen_u(G, seed, u, SC_GEN_D_ROT), sc_gen_u(G, seed, u, SC_GEN_D_ROT + 1),
                                           sc_gen_u(G, seed, u, SC_GEN_D_ROT + 2));
            const float wrapRate = 0.3f;
            const int32_t id0 = G->first + u * n;
            for (int s = 0; s < n; s++) {
                const int k = s % G->mix.nkinds;
                if (s > 0) {
                    const uint32_t d = SC_GEN_D_ROT + 3u * (uint32_t)s;
                    rot = sc_slerp(rot, sc_random_rotation(sc_gen_u(G, seed, u, d), sc_gen_u(G, seed, u, d + 1),
                                                           sc_gen_u(G, seed, u, d + 2)),
                                   wrapRate);
                    const sc_f3 dPos = sc_rotate(sc_up(), rot) * -(G->prevRadius[k] + G->mix.radius[k]);
                    pos = pos + dPos;
                }
                sc_gen_put(&out[s], id0 + s, &G->mix, k, pos, rot, box);
            }
            for (int s = 1; s < n; s++) sc_gen_link(&out[s - 1], &out[s], G->link);
            break;
        }
        default: break;
    }
}

// Validates scene groups and fills gg (first particle of each group, mixes,
// the chains' type-(t-1) radii, streams, the reference's count-based radius
// for a Fibonacci shell given radius <= 0); returns the particle total, or
// -1 with *why set.  Host code.
static inline int64_t sc_gen_prepare(const sc_scene_group *g, int32_t ng, const sc_type_info *types, int32_t ntypes,
                                     sc_gen_group *gg, const char **why) {
    int64_t total = 0;
    for (int32_t i = 0; i < ng; i++) {
        const sc_scene_group &a = g[i];
        sc_gen_group &G = gg[i];
        memset(&G, 0, sizeof G);
        const bool compound = a.kind == SC_SCENE_COMPLEXES || a.kind == SC_SCENE_WRAPPED_CHAINS;
        if (a.kind < SC_SCENE_UNIFORM_BOX || a.kind > SC_SCENE_WRAPPED_CHAINS) { *why = "unknown scene group kind"; return -1; }
        if (a.count < 0) { *why = "negative group count"; return -1; }
        if (compound && (a.unit < 1 || a.unit > SC_SCENE_MAX_UNIT)) { *why = "complex / chain size outside 1..64"; return -1; }
        if (sc_gen_make_mix(&G.mix, a.kinds, a.fractions, a.nkinds, types, ntypes)) {
            *why = "a group's mix needs 1 to 4 kinds of the type table, weights >= 0";
            return -1;
        }
        if (!(a.radius >= 0.0f) && a.kind != SC_SCENE_FIBONACCI_SHELL) { *why = "negative group radius"; return -1; }
        if (a.kind == SC_SCENE_COMPLEXES && !(a.spacing > 0.0f)) { *why = "complex spacing must be > 0"; return -1; }
        G.kind = a.kind;
        G.count = a.count;
        G.unit = compound ? a.unit : 1;
        G.first = (int32_t)total;
        for (int k = 0; k < 3; k++) G.center[k] = a.center[k];
        G.radius = a.radius;
        G.spacing = a.spacing;
        for (int k = 0; k < 4; k++) G.rot[k] = a.rot[k];
        G.link = a.link_type;
        G.stream = SC_GEN_STREAM_SCENE + (uint32_t)i;
        if (a.kind == SC_SCENE_WRAPPED_CHAINS) {
            for (int k = 0; k < G.mix.nkinds; k++) {
                const int t = G.mix.kind[k] - 1;  // particle_setup.cuh:99 steps by the radius of type id t-1
                if (t < 0 || t >= ntypes) { *why = "a chain member type needs type id t-1 in the table"; return -1; }
                G.prevRadius[k] = types[t].radius;
            }
        }
        if (a.kind == SC_SCENE_FIBONACCI_SHELL && !(a.radius > 0.0f))  // particle_setup.cuh:210
            G.radius = (float)(sqrt(a.count / 1000.0 * pow(G.mix.radius[0] / 2.5, 2.0)) * 40.0);
        total += sc_gen_group_particles(a.kind, a.count, a.unit);
        if (total > 0x7fffffff) { *why = "scene larger than 2^31 particles"; return -1; }
    }
    return total;
}
