// scport.cpp -- CPU restatement of spatial_cell_sim's step.
//
// TEST INFRASTRUCTURE ONLY: what the sm_103a step is checked against (tests/,
// __graft_entry__.smoke()) and the timed CPU baseline of bench.py.  Nothing
// in the product links or calls it.
//
// It restates the reference kernels (spatial_cell_sim/src/grid.cuh,
// dynamics.cuh, interactions.cuh, metabolites.cuh) over the reference's own
// array-of-structs layout (256-byte Particle, 304-byte MetabolicParticle),
// kernel by kernel, in the launch order of main.cu:347-661, with the same
// double-buffer semantics (every neighbour kernel reads the current array and
// writes a cleared next array).  Floating-point expressions are evaluated in
// the reference's order and types (including its implicit double-precision
// literals); elementary functions, the Philox noise and binary16 conversion
// come from scmath.h.  Parity of this file with the reference's own code is
// checked by tests/test_oracle_ref.py against oracle/_ref (the reference
// compiled for the host) and by the committed golden vectors.
//
// Each thread index of a reference kernel is one loop iteration here; the
// double-buffered kernels are independent per index and run under OpenMP.
// polymerize (in place, cross-slot writes) runs sequentially in slot order.
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "scmath.h"
#include "spatialcell.h"
#include "sc_gen.h"

// The state's own single-precision scalar (the ABI layouts stay float in
// both builds below).
typedef float sc_single;

#if defined(SC_PORT_FP64)
// The FP64 build (oracle/scport64.cpp): every floating-point quantity of the
// step is a double -- state, temporaries, the reference's double-precision
// expressions as they are -- with oracle/scmath64.h's vector / quaternion
// helpers and the C library's double elementary functions.  The noise
// draws, the rules and the load / export records stay the reference's
// single-precision values (converted at the boundary).
#include <math.h>
#include "scmath64.h"
#define sc_f2 sc_d2
#define sc_f3 sc_d3
#define sc_f4 sc_d4
#define sc_make_f3 sc_make_d3
#define sc_make_f4 sc_make_d4
#define sc_up sc_d_up
#define sc_right sc_d_right
#define sc_forward sc_d_forward
#define sc_zero3 sc_d_zero3
#define sc_qid sc_d_qid
#define sc_normsq3 sc_d_normsq3
#define sc_normsq4 sc_d_normsq4
#define sc_norm3 sc_d_norm3
#define sc_safe_cross sc_d_safe_cross
#define sc_qmul sc_d_qmul
#define sc_angle3 sc_d_angle3
#define sc_quat sc_d_quat
#define sc_quat_from_to sc_d_quat_from_to
#define sc_qinv sc_d_qinv
#define sc_slerp sc_d_slerp
#define sc_random_rotation sc_d_random_rotation
#define sc_rotate sc_d_rotate
#define sc_image3 sc_d_image3
#define sc_wrap3 sc_d_wrap3
#define sc_reflect3 sc_d_reflect3
#define sc_grid_idx sc_d_grid_idx
#define sc_powf pow
#define float double
#define fabsf fabs
#define fminf fmin
#define fmaxf fmax
#define sqrtf sqrt
#endif

#if defined(_OPENMP)
#include <omp.h>
#define SC_OMP_FOR _Pragma("omp parallel for schedule(dynamic, 256)")
#else
#define SC_OMP_FOR
#endif

namespace {

const int32_t kActive = SC_PARTICLE_FLAG_ACTIVE;
const uint32_t kMaxKey = 0xFFFFFFFFu;

// The reference's Particle (types.cuh:173-222), field for field.
struct PP {
    int32_t id, type, flags;
    int8_t state;
    int32_t lscs;
    float radius;
    int8_t hydro;
    sc_f3 pos;
    sc_f4 rot;
    sc_f3 vel;
    sc_f3 posNoise;
    sc_f4 angVel;
    sc_f4 angNoise;
    int32_t nb;
    sc_interaction bonds[SC_MAX_ACTIVE_INTERACTIONS];
    int32_t spoly;
    sc_f4 dbg;
};
struct PM : PP {
    float m[SC_AOS_NUM_METABOLITES];
};
#if !defined(SC_PORT_FP64)
static_assert(sizeof(PP) == 256 && offsetof(PP, pos) == 28 && offsetof(PP, rot) == 48, "Particle layout");
static_assert(offsetof(PP, angVel) == 96 && offsetof(PP, nb) == 128 && offsetof(PP, dbg) == 240, "Particle layout");
static_assert(sizeof(PM) == 304 && offsetof(PM, m) == 256, "MetabolicParticle layout");
static_assert(sizeof(PP) == sizeof(sc_particle) && sizeof(PM) == sizeof(sc_metabolic_particle), "ABI layout");

// State records in and out: the reference's layout byte for byte.
void put_particles(PP *dst, const sc_particle *src, int n) { memcpy((void *)dst, src, (size_t)n * sizeof(PP)); }
void put_metabolic(PM *dst, const sc_metabolic_particle *src, int n) { memcpy((void *)dst, src, (size_t)n * sizeof(PM)); }
void get_particles(sc_particle *dst, const PP *src, int n) { memcpy(dst, (const void *)src, (size_t)n * sizeof(PP)); }
void get_metabolic(sc_metabolic_particle *dst, const PM *src, int n) { memcpy(dst, (const void *)src, (size_t)n * sizeof(PM)); }
#else
// State records in and out: every field converted between the reference's
// single-precision layout and this build's doubles.
void put_particle(PP &d, const sc_particle &r) {
    d.id = r.id; d.type = r.type; d.flags = r.flags; d.state = r.state; d.lscs = r.last_state_change_step;
    d.radius = r.radius; d.hydro = r.hydrophobic;
    d.pos = sc_make_d3(r.pos[0], r.pos[1], r.pos[2]);
    d.rot = sc_make_d4(r.rot[0], r.rot[1], r.rot[2], r.rot[3]);
    d.vel = sc_make_d3(r.velocity[0], r.velocity[1], r.velocity[2]);
    d.posNoise = sc_make_d3(r.pos_noise[0], r.pos_noise[1], r.pos_noise[2]);
    d.angVel = sc_make_d4(r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2], r.angular_velocity[3]);
    d.angNoise = sc_make_d4(r.angular_noise[0], r.angular_noise[1], r.angular_noise[2], r.angular_noise[3]);
    d.nb = r.n_active_interactions;
    memcpy(d.bonds, r.interactions, sizeof d.bonds);
    d.spoly = r.scheduled_polymerization;
    d.dbg = sc_make_d4(r.debug_vector[0], r.debug_vector[1], r.debug_vector[2], r.debug_vector[3]);
}
void get_particle(sc_particle &r, const PP &d) {
    memset(&r, 0, sizeof r);
    r.id = d.id; r.type = d.type; r.flags = d.flags; r.state = d.state; r.last_state_change_step = d.lscs;
    r.radius = (sc_single)d.radius; r.hydrophobic = d.hydro;
    const sc_single v[] = {(sc_single)d.pos.x, (sc_single)d.pos.y, (sc_single)d.pos.z, (sc_single)d.rot.x,
                           (sc_single)d.rot.y, (sc_single)d.rot.z, (sc_single)d.rot.w, (sc_single)d.vel.x,
                           (sc_single)d.vel.y, (sc_single)d.vel.z, (sc_single)d.posNoise.x, (sc_single)d.posNoise.y,
                           (sc_single)d.posNoise.z, (sc_single)d.angVel.x, (sc_single)d.angVel.y,
                           (sc_single)d.angVel.z, (sc_single)d.angVel.w, (sc_single)d.angNoise.x,
                           (sc_single)d.angNoise.y, (sc_single)d.angNoise.z, (sc_single)d.angNoise.w,
                           (sc_single)d.dbg.x, (sc_single)d.dbg.y, (sc_single)d.dbg.z, (sc_single)d.dbg.w};
    memcpy(r.pos, v, 3 * sizeof(sc_single));
    memcpy(r.rot, v + 3, 4 * sizeof(sc_single));
    memcpy(r.velocity, v + 7, 3 * sizeof(sc_single));
    memcpy(r.pos_noise, v + 10, 3 * sizeof(sc_single));
    memcpy(r.angular_velocity, v + 13, 4 * sizeof(sc_single));
    memcpy(r.angular_noise, v + 17, 4 * sizeof(sc_single));
    memcpy(r.debug_vector, v + 21, 4 * sizeof(sc_single));
    r.n_active_interactions = d.nb;
    memcpy(r.interactions, d.bonds, sizeof d.bonds);
    r.scheduled_polymerization = d.spoly;
}
void put_particles(PP *dst, const sc_particle *src, int n) { for (int i = 0; i < n; i++) put_particle(dst[i], src[i]); }
void put_metabolic(PM *dst, const sc_metabolic_particle *src, int n) {
    for (int i = 0; i < n; i++) {
        put_particle(dst[i], src[i].p);
        for (int k = 0; k < SC_AOS_NUM_METABOLITES; k++) dst[i].m[k] = src[i].metabolites[k];
    }
}
void get_particles(sc_particle *dst, const PP *src, int n) { for (int i = 0; i < n; i++) get_particle(dst[i], src[i]); }
void get_metabolic(sc_metabolic_particle *dst, const PM *src, int n) {
    for (int i = 0; i < n; i++) {
        memset(&dst[i], 0, sizeof dst[i]);
        get_particle(dst[i].p, src[i]);
        for (int k = 0; k < SC_AOS_NUM_METABOLITES; k++) dst[i].metabolites[k] = (sc_single)src[i].m[k];
    }
}
#endif

// Particle(...) constructor of types.cuh:192-221
PP make_particle(int id, int type, float radius, int8_t hydro, sc_f3 pos, sc_f4 rot) {
    PP p;
    memset(&p, 0, sizeof p);
    p.id = id; p.type = type; p.flags = kActive; p.state = 0; p.lscs = -1;
    p.radius = radius; p.hydro = hydro; p.pos = pos; p.rot = rot;
    p.vel = sc_zero3(); p.posNoise = sc_zero3(); p.angVel = sc_qid(); p.angNoise = sc_qid();
    p.nb = 0; p.spoly = -1; p.dbg = sc_make_f4(0, 0, 0, 0);
    return p;
}

sc_rule zero_rule() { sc_rule r; memset(&r, 0, sizeof r); return r; }
sc_f4 rule_ori(const sc_rule &r) { return sc_make_f4(r.relative_orientation[0], r.relative_orientation[1], r.relative_orientation[2], r.relative_orientation[3]); }
sc_f3 rule_pos(const sc_rule &r) { return sc_make_f3(r.relative_position[0], r.relative_position[1], r.relative_position[2]); }

// interactions.cuh:186-189
inline bool order(const PP &a, const PP &b) { return a.type < b.type || (a.type == b.type && a.id < b.id); }
// interactions.cuh:191-197
inline sc_f4 target_rel_ori(const PP &p, const PP &tp, sc_f4 q) {
    return order(p, tp) ? sc_qmul(tp.rot, sc_qinv(q)) : sc_qmul(tp.rot, q);
}
// interactions.cuh:199-213
inline sc_f3 relaxed_rel_pos(const PP &p, const PP &tp, sc_f4 tro, sc_f4 trpr, float dist) {
    sc_f3 r = order(p, tp) ? -sc_rotate(sc_up(), sc_qmul(tp.rot, sc_qmul(sc_qinv(tro), trpr)))
                           : sc_rotate(sc_up(), sc_qmul(tp.rot, trpr));
    r *= dist;
    r += tp.pos;
    return r;
}

}  // namespace

struct scp_sim {
    sc_config cfg;
    int ngrid = 2, nbits = 1;
    size_t cells = 8;
    int N = 0, Nm = 0, S = 10;
    std::vector<PP> p, pn;
    std::vector<PM> m, mn;
    std::vector<uint32_t> keyP, keyM, permP, permM, rangesP, rangesM;
    std::vector<sc_type_info> types;
    std::vector<sc_rule> flat;      // id-indexed (flattenComplexificationInfo)
    std::vector<int32_t> pidx;      // partner index, 2 * (max rule id + 1)
    std::vector<sc_rule> prules;    // partner-mapped rules
    int nActive = 0, lastActive = -1, nextId = 0, nActiveM = 0, step = 0;
    bool periodic = false;   // periodic box extension (cfg.periodic)
    int nUsed = 2;           // cells per axis that hold positions, ceil(simSize / cell)
    float cellSize = 1.0f;   // cell width: the configured size, in a periodic box simSize / nUsed

    const sc_rule &rule(int id) const {
        static const sc_rule z = zero_rule();
        return (id >= 0 && (size_t)id < flat.size()) ? flat[(size_t)id] : z;
    }
    uint32_t cell_key(uint32_t gx, uint32_t gy, uint32_t gz) const {
        return (gx << (2 * nbits)) | (gy << nbits) | gz;
    }
    // cells per axis the cell index clamps to: the power-of-two grid of
    // config.cuh:65-74, or in a periodic box the cells the box spans
    int idx_limit() const { return periodic ? nUsed : ngrid; }
    uint32_t key_of(sc_f3 pos) const {
        float c = cellSize;
        int n = idx_limit();
        return cell_key(sc_grid_idx(pos.x, c, n), sc_grid_idx(pos.y, c, n), sc_grid_idx(pos.z, c, n));
    }
    // position of a neighbour as seen from pos (its nearest periodic image)
    sc_f3 img(sc_f3 t, sc_f3 pos) const { return periodic ? sc_image3(t, pos, cfg.sim_size) : t; }
    // Visits the 27 (clamped) cells around pos in the reference's gx, gy, gz
    // order; per cell calls f(key).
    template <class F>
    void cells27(sc_f3 pos, F &&f) const {
        float c = cellSize;
        int n = idx_limit();
        int cx = (int)sc_grid_idx(pos.x, c, n), cy = (int)sc_grid_idx(pos.y, c, n), cz = (int)sc_grid_idx(pos.z, c, n);
        if (periodic) {
            // offsets -1, 0, +1 per axis, wrapped (the order of a periodic scan)
            for (int ox = -1; ox <= 1; ox++)
                for (int oy = -1; oy <= 1; oy++)
                    for (int oz = -1; oz <= 1; oz++)
                        f(cell_key((uint32_t)((cx + ox + n) % n), (uint32_t)((cy + oy + n) % n),
                                   (uint32_t)((cz + oz + n) % n)));
            return;
        }
        for (int gx = std::max(cx - 1, 0); gx <= std::min(cx + 1, ngrid - 1); gx++)
            for (int gy = std::max(cy - 1, 0); gy <= std::min(cy + 1, ngrid - 1); gy++)
                for (int gz = std::max(cz - 1, 0); gz <= std::min(cz + 1, ngrid - 1); gz++)
                    f(cell_key((uint32_t)gx, (uint32_t)gy, (uint32_t)gz));
    }
    template <class F>
    void scan(const std::vector<uint32_t> &ranges, sc_f3 pos, F &&f) const {
        cells27(pos, [&](uint32_t k) {
            for (uint32_t j = ranges[2 * (size_t)k]; j < ranges[2 * (size_t)k + 1]; j++) f((int)j);
        });
    }
};

namespace {

bool outside_cube(sc_f3 d, float lim) { return fabsf(d.x) > lim || fabsf(d.y) > lim || fabsf(d.z) > lim; }

// ---- grid.cuh:34-139: keys, stable sort, cell ranges ------------------------
template <class T>
void sort_items(scp_sim &s, std::vector<T> &cur, std::vector<T> &nxt, std::vector<uint32_t> &key,
                std::vector<uint32_t> &perm, std::vector<uint32_t> &ranges, int n) {
    key.assign((size_t)n, 0);
    SC_OMP_FOR
    for (int i = 0; i < n; i++) key[i] = (cur[i].flags & kActive) ? s.key_of(cur[i].pos) : kMaxKey;
    // stable LSD counting sort (same order as CUB's stable radix sort)
    std::vector<uint32_t> idx((size_t)n), tmp((size_t)n);
    for (int i = 0; i < n; i++) idx[i] = (uint32_t)i;
    for (int shift = 0; shift < 32; shift += 8) {
        std::vector<size_t> cnt(257, 0);
        for (int i = 0; i < n; i++) cnt[((key[idx[i]] >> shift) & 0xFF) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (int i = 0; i < n; i++) tmp[cnt[(key[idx[i]] >> shift) & 0xFF]++] = idx[i];
        idx.swap(tmp);
    }
    perm = idx;
    std::vector<uint32_t> sk((size_t)n);
    SC_OMP_FOR
    for (int i = 0; i < n; i++) { nxt[i] = cur[idx[i]]; sk[i] = key[idx[i]]; }
    cur.swap(nxt);
    key.swap(sk);
    ranges.assign(s.cells * 2, 0);
    for (int i = 0; i < n; i++) {
        uint32_t k = key[i];
        if (k == kMaxKey) continue;
        if (i == 0 || key[i - 1] != k) ranges[2 * (size_t)k] = (uint32_t)i;
        if (i == n - 1 || key[i + 1] != k) ranges[2 * (size_t)k + 1] = (uint32_t)(i + 1);
    }
}

template <class T>
void clear_tail(std::vector<T> &v, int from) {
    if ((size_t)from < v.size()) memset((void *)&v[(size_t)from], 0, (v.size() - (size_t)from) * sizeof(T));
}

// ---- dynamics.cuh:19-154 move (its neighbour loop has no live effect) ---------
template <class T>
void move_items(std::vector<T> &cur, std::vector<T> &nxt, int n) {
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        T p = cur[i];
        if (p.flags & kActive) { p.dbg.x = 0; p.dbg.y = 0; p.dbg.z = 0; }
        nxt[i] = p;
    }
    clear_tail(nxt, n);
    cur.swap(nxt);
}

// ---- dynamics.cuh:156-215 brownianMovementAndRotation -----------------------
template <class T>
void brownian(const scp_sim &s, std::vector<T> &items, int n, float scale, uint32_t su, uint32_t sn) {
    const uint64_t seed = s.cfg.seed;
    const uint32_t step = (uint32_t)s.step;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        T &p = items[i];
        if (!(p.flags & kActive)) continue;
        uint32_t id = (uint32_t)p.id;
        sc_f4 r1 = sc_random_rotation(sc_uniform(seed, su, id, step, 0), sc_uniform(seed, su, id, step, 1),
                                      sc_uniform(seed, su, id, step, 2));
        float nrm = sc_normal(seed, sn, id, step, 0);
        float mag = (float)((double)(fabsf(nrm) * scale) / fmax((double)p.radius / 2.5, 1.0));
        p.posNoise = sc_rotate(sc_up(), r1) * mag;
        sc_f4 r2 = sc_random_rotation(sc_uniform(seed, su, id, step, 3), sc_uniform(seed, su, id, step, 4),
                                      sc_uniform(seed, su, id, step, 5));
        float t = (float)((double)s.cfg.rotation_noise_scale / ((double)p.radius / 2.5));
        p.angNoise = sc_slerp(p.angNoise, r2, t);
    }
}

// ---- dynamics.cuh:217-242 applyNoise -----------------------------------------
template <class T>
void apply_noise(std::vector<T> &items, int n) {
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        T &p = items[i];
        if (!(p.flags & kActive)) continue;
        p.vel += p.posNoise;
        p.posNoise = sc_zero3();
        p.angVel = sc_qmul(p.angNoise, p.angVel);
        p.angNoise = sc_qid();
    }
}

// ---- dynamics.cuh:244-282 applyVelocities ------------------------------------
template <class T>
void apply_velocities(const scp_sim &s, std::vector<T> &items, int n, float f) {
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        T &p = items[i];
        if (!(p.flags & kActive)) continue;
        p.pos = s.periodic ? sc_wrap3(p.pos + p.vel * f, s.cfg.sim_size)
                           : (s.cfg.walls ? sc_reflect3(p.pos + p.vel * f, s.cfg.sim_size)
                                          : clamp(p.pos + p.vel * f, 0.0f, s.cfg.sim_size));
        p.vel *= s.cfg.velocity_decay;
        p.rot = sc_qmul(sc_slerp(sc_qid(), p.angVel, f), p.rot);
        p.rot /= length(p.rot);
        p.angVel = sc_slerp(p.angVel, sc_qid(), 1.0f - s.cfg.angular_velocity_decay);
    }
}

// ---- dynamics.cuh:288-402 coordinateNoise ------------------------------------
void coordinate_noise(scp_sim &s, float frac) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive) || p.nb < 1) { s.pn[i] = p; continue; }
        sc_f3 dPN = sc_zero3();
        sc_f4 dAN = sc_qid();
        float w = 0.0f;
        s.scan(s.rangesP, p.pos, [&](int j) {
            if (j == i) return;
            const PP &tp = cur[j];
            if (!(tp.flags & kActive)) return;
            sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
            if (outside_cube(delta, lim)) return;
            for (int k = 0; k < p.nb; k++) {
                const sc_interaction &it = p.bonds[k];
                if (it.type < 10 && frac > 0.25f) continue;
                if (it.partner_id == tp.id) {
                    float pMag = length(p.posNoise);
                    dPN += (tp.posNoise - p.posNoise) * 0.9f * tp.radius / (p.radius + tp.radius) * 1.0f;
                    dPN *= fmaxf(length(dPN), pMag) / length(dPN);
                    dAN = sc_slerp(dAN, sc_qmul(sc_qinv(p.angNoise), tp.angNoise),
                                   0.9f * tp.radius / (p.radius + tp.radius) * 1.0f);
                    w += 1.0f;
                }
            }
        });
        p.posNoise += dPN / fmaxf(w, 1.0f);
        p.angNoise = sc_qmul(sc_slerp(sc_qid(), dAN, 1.0f / fmaxf(w, 1.0f)), p.angNoise);
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// ---- dynamics.cuh:405-822 relax -------------------------------------------------
void relax(scp_sim &s) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    const float flex = SC_PI_REF / 8;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive)) { s.pn[i] = p; continue; }
        sc_f3 dV = sc_zero3();
        sc_f4 dAV = sc_qid();
        sc_f3 phobPos = sc_zero3();
        float phobSum = 0.0f;
        float w = 0.0f;
        const sc_f3 up = sc_rotate(sc_up(), p.rot);
        const sc_f3 nextUp = sc_rotate(up, p.angVel);
        s.scan(s.rangesP, p.pos, [&](int j) {
            if (j == i) return;
            const PP &tp0 = cur[j];
            if (!(tp0.flags & kActive)) return;
            PP timg;
            const PP *tq = &tp0;
            if (s.periodic) { timg = tp0; timg.pos = s.img(tp0.pos, p.pos); tq = &timg; }
            const PP &tp = *tq;
            sc_f3 delta = tp.pos - p.pos;
            if (outside_cube(delta, lim)) return;
            sc_f3 nd = normalize(delta);
            float dist = sc_norm3(delta);
            float idist = p.radius + tp.radius;
            sc_f3 tup = sc_rotate(sc_up(), tp.rot);
            sc_f3 nextTup = sc_rotate(tup, p.angVel);
            if (p.hydro > 0 || tp.hydro > 0) {
                float s2 = p.radius + tp.radius;
                if ((double)dist <= (double)s2 + 0.8 * (double)s2 * 0.5) {
                    if (p.hydro == SC_POLAR && tp.hydro == SC_POLAR) {
                        sc_f3 pPV = -nextUp * p.radius + p.pos + p.vel;
                        sc_f3 tpPV = -nextTup * tp.radius + tp.pos + tp.vel;
                        float L = length(tpPV - pPV) / (p.radius + tp.radius);
                        float attr = (float)(fmin(fmax((double)L, 1e-6), (double)2.0f) / (double)2.0f);
                        w += 1.0f;
                        dV += (tpPV - pPV) * 0.05f * attr * 1.0f;
                        float pap = sc_powf(fminf(1.0f / fmaxf(L, 1e-6f), 10.0f) / 10.0f, 0.2f);
                        phobSum += pap;
                        phobPos += tpPV * pap;
                    }
                }
            }
            bool partners = false;
            for (int k = 0; k < p.nb; k++) {
                const sc_interaction it = p.bonds[k];
                if (it.partner_id != tp.id) continue;
                partners = true;
                if (it.type >= 10) {
                    const sc_rule &pii = s.rule(it.type);
                    sc_f4 ro = rule_ori(pii);
                    sc_f3 rp = rule_pos(pii);
                    sc_f4 rro = sc_qmul(sc_qinv(sc_qmul(p.angVel, p.rot)), sc_qmul(tp.angVel, target_rel_ori(p, tp, ro)));
                    sc_f4 orro = sc_qmul(sc_qinv(sc_qmul(tp.angVel, tp.rot)), sc_qmul(p.angVel, target_rel_ori(tp, p, ro)));
                    dAV = sc_slerp(dAV, sc_qmul(sc_slerp(rro, orro, 0.5f), rro), 0.9f * tp.radius / (p.radius + tp.radius));
                    sc_f3 rrp = order(p, tp) ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(tp.angVel, tp.rot)))
                                             : sc_rotate(rp, sc_qmul(tp.angVel, tp.rot));
                    rrp += tp.pos;
                    sc_f3 orrp = order(tp, p) ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(p.angVel, p.rot)))
                                              : sc_rotate(rp, sc_qmul(p.angVel, p.rot));
                    orrp += p.pos;
                    w += 1.0f;
                    sc_f3 pDV = (rrp + tp.vel - (p.pos + p.vel)) * 0.9f * tp.radius / (p.radius + tp.radius) * 1.0f;
                    sc_f3 tpDV = (orrp + p.vel - (tp.pos + tp.vel)) * 0.9f * p.radius / (p.radius + tp.radius) * 1.0f;
                    dV += (pDV - (pDV + tpDV) / 2.0f) * 0.9f * p.radius / (p.radius + tp.radius) * 1.0f;
                }
                if (it.type == 0) {
                    sc_f4 trod = sc_qmul(sc_quat(sc_up(), -SC_PI_REF / 6), sc_quat(sc_right(), SC_PI_REF / 6));
                    p.rot = sc_slerp(p.rot, target_rel_ori(p, tp, trod), 0.2f);
                    sc_f4 trpr = sc_quat(sc_forward(), -SC_PI_REF / 6);
                    sc_f3 rrp = relaxed_rel_pos(p, tp, trod, trpr, idist);
                    p.dbg.x = (float)((double)p.dbg.x + (double)(rrp.x - p.pos.x) * (1.0 - (double)0.2f));
                    p.dbg.y = (float)((double)p.dbg.y + (double)(rrp.y - p.pos.y) * (1.0 - (double)0.2f));
                    p.dbg.z = (float)((double)p.dbg.z + (double)(rrp.z - p.pos.z) * (1.0 - (double)0.2f));
                } else if (it.type == SC_INTERACTION_TYPE_CHAIN) {
                    sc_f3 nnd = normalize(tp.pos + tp.vel - (p.pos + p.vel));
                    bool fwd = it.group == SC_INTERACTION_GROUP_FORWARD;
                    dAV = sc_slerp(dAV, sc_quat_from_to(nextUp, (fwd ? -1.0f : 1.0f) * nnd),
                                   0.9f * tp.radius / (p.radius + tp.radius));
                    sc_f3 relUp = (fwd ? 1.0f : -1.0f) * nextTup;
                    sc_f3 axis = sc_safe_cross(relUp, -nnd);
                    float ang = sc_angle3(relUp, -nnd);
                    sc_f3 rrp = sc_rotate(relUp, sc_quat(axis, fminf(fmaxf(ang, -flex), flex)));
                    rrp *= idist;
                    rrp += tp.pos;
                    sc_f3 oUp = (fwd ? -1.0f : 1.0f) * nextUp;
                    sc_f3 oaxis = sc_safe_cross(oUp, nnd);
                    float oang = sc_angle3(oUp, nnd);
                    sc_f3 orrp = sc_rotate(oUp, sc_quat(oaxis, fminf(fmaxf(oang, -flex), flex)));
                    orrp *= idist;
                    orrp += p.pos;
                    w += 1.0f;
                    sc_f3 pDV = (rrp + tp.vel - (p.pos + p.vel)) * 0.9f * tp.radius / (p.radius + tp.radius) * 1.0f;
                    sc_f3 tpDV = (orrp + p.vel - (tp.pos + tp.vel)) * 0.9f * p.radius / (p.radius + tp.radius) * 1.0f;
                    dV += (pDV - (pDV + tpDV) / 2.0f) * 0.9f * p.radius / (p.radius + tp.radius) * 1.0f;
                    p.dbg.x = (float)((double)p.dbg.x + (double)(rrp.x - p.pos.x) * (1.0 - (double)0.9f));
                    p.dbg.y = (float)((double)p.dbg.y + (double)(rrp.y - p.pos.y) * (1.0 - (double)0.9f));
                    p.dbg.z = (float)((double)p.dbg.z + (double)(rrp.z - p.pos.z) * (1.0 - (double)0.9f));
                }
            }
            if (!partners) {
                float cd = p.radius + tp.radius;
                if (dist < cd) {
                    w += 1.0f;
                    dV += (tp.pos - nd * cd + tp.vel - (p.pos + p.vel)) * 0.9f * tp.radius / (p.radius + tp.radius) * 1.0f;
                }
            }
        });
        p.vel += dV / fmaxf(w, 1.0f);
        p.angVel = sc_qmul(sc_slerp(sc_qid(), dAV, 1.0f / fmaxf(w, 1.0f)), p.angVel);
        if (phobSum > 0.0f) {
            sc_f3 dir = normalize(phobPos / phobSum - (p.pos + p.vel));
            p.angVel = sc_slerp(p.angVel, sc_quat_from_to(-up, dir), 0.2f);
        }
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// (double)(r_p + r_t) + 0.8 * (double)r_p rounded to float (metabolites.cuh:198)
inline float metab_collision_dist(float rp, float rt) { return (float)((double)(rp + rt) + 0.8 * (double)rp); }

// ---- metabolites.cuh:140-264 relaxMetabolicParticles -----------------------
void relax_metab(scp_sim &s) {
    const int n = s.nActiveM;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PM> &cur = s.m;
    const std::vector<PP> &parts = s.p;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PM p = cur[i];
        if (!(p.flags & kActive)) { s.mn[i] = p; continue; }
        sc_f3 dV = sc_zero3();
        float w = 0.0f;
        s.cells27(p.pos, [&](uint32_t key) {
            for (uint32_t j = s.rangesM[2 * (size_t)key]; j < s.rangesM[2 * (size_t)key + 1]; j++) {
                if ((int)j == i) continue;
                const PM &tp = cur[j];
                if (!(tp.flags & kActive)) continue;
                sc_f3 tpos = s.img(tp.pos, p.pos);
                sc_f3 delta = tpos - p.pos;
                if (outside_cube(delta, lim)) continue;
                sc_f3 nd = normalize(delta);
                float dist = sc_norm3(delta);
                float cd = metab_collision_dist(p.radius, tp.radius);
                if (dist <= cd) {
                    w += 1.0f;
                    dV += (tpos - nd * cd + tp.vel - (p.pos + p.vel)) * 0.9f * 1.0f;
                }
            }
            for (uint32_t j = s.rangesP[2 * (size_t)key]; j < s.rangesP[2 * (size_t)key + 1]; j++) {
                const PP &tp = parts[j];
                if (!(tp.flags & kActive) || tp.type != SC_PARTICLE_TYPE_LIPID) continue;
                sc_f3 tpos = s.img(tp.pos, p.pos);
                sc_f3 delta = tpos - p.pos;
                if (outside_cube(delta, lim)) continue;
                sc_f3 nd = normalize(delta);
                float dist = sc_norm3(delta);
                float cd = metab_collision_dist(p.radius, tp.radius);
                if (dist <= cd) {
                    w += 2.0f;
                    dV += (tpos - nd * cd + tp.vel - (p.pos + p.vel)) * 0.9f * 2.0f;
                }
            }
        });
        p.vel += dV / fmaxf(w, 1.0f);
        s.mn[i] = p;
    }
    clear_tail(s.mn, n);
    s.m.swap(s.mn);
}

// ---- metabolites.cuh:266-350 relaxMetabolicParticlePartners -----------------
void relax_partners(scp_sim &s) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    const std::vector<PM> &met = s.m;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive) || p.type != SC_PARTICLE_TYPE_LIPID) { s.pn[i] = p; continue; }
        sc_f3 dV = sc_zero3();
        float w = 0.0f;
        s.scan(s.rangesM, p.pos, [&](int j) {
            const PM &tp = met[j];
            if (!(tp.flags & kActive)) return;
            sc_f3 tpos = s.img(tp.pos, p.pos);
            sc_f3 delta = tpos - p.pos;
            if (outside_cube(delta, lim)) return;
            sc_f3 nd = normalize(delta);
            float dist = sc_norm3(delta);
            float cd = metab_collision_dist(p.radius, tp.radius);
            if (dist <= cd) {
                w += 2.0f;
                dV += (tpos - nd * cd + tp.vel - (p.pos + p.vel)) * 0.9f * 2.0f;
            }
        });
        p.vel += dV / fmaxf(w, 1.0f);
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// Alignment tests shared by complexify and transitionInteractions
// (interactions.cuh:319-324, 438-443).
inline void alignment(const PP &p, const PP &tp, sc_f3 up, sc_f3 tup, sc_f3 delta, const sc_rule &r, float *oa,
                      float *rpa) {
    bool ord = order(p, tp);
    sc_f4 ro = rule_ori(r);
    sc_f3 rp = rule_pos(r);
    *oa = ord ? dot(sc_rotate(up, ro), tup) : dot(sc_rotate(tup, ro), up);
    *rpa = ord ? dot(sc_rotate(rp, p.rot), delta) / sc_normsq3(delta) : dot(sc_rotate(rp, tp.rot), -delta) / sc_normsq3(delta);
}
inline bool states_match(const PP &p, const PP &tp, const sc_rule &r) {
    return order(p, tp) ? ((r.first_partner_state < 0 || r.first_partner_state == p.state) &&
                           (r.second_partner_state < 0 || r.second_partner_state == tp.state))
                        : ((r.second_partner_state < 0 || r.second_partner_state == p.state) &&
                           (r.first_partner_state < 0 || r.first_partner_state == tp.state));
}
inline bool group_active(const PP &a, int group) {
    for (int k = 0; k < a.nb; k++)
        if (a.bonds[k].group == group) return true;
    return false;
}

// The binding draw of a rule with a probability (extension; the reference's
// rules always pass).
inline bool bind_draw(const scp_sim &s, const sc_rule &r, int pid, int tid, int step) {
    return !r.use_probability || sc_bind_uniform(s.cfg.seed, r.id, pid, tid, step) < r.probability;
}

void complexify_claim(scp_sim &s, int step);

// ---- interactions.cuh:216-346 complexify -------------------------------------
// step: the kernel's step argument (-1 in the start-up sequence); it only
// keys the binding draws of rules with a probability.
void complexify(scp_sim &s, int step) {
    if (s.cfg.pair_claim) { complexify_claim(s, step); return; }
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive)) { s.pn[i] = p; continue; }
        const sc_f3 up = sc_rotate(sc_up(), p.rot);
        int cs = 0, ce = 0;
        if (p.type >= 0 && (size_t)p.type * 2 + 1 < s.pidx.size()) { cs = s.pidx[p.type * 2]; ce = s.pidx[p.type * 2 + 1]; }
        if (cs < ce) {
            s.scan(s.rangesP, p.pos, [&](int j) {
                if (j == i) return;
                const PP &tp = cur[j];
                if (!(tp.flags & kActive)) return;
                sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
                if (outside_cube(delta, lim)) return;
                sc_f3 tup = sc_rotate(sc_up(), tp.rot);
                for (int k = cs; k < ce; k++) {
                    if (p.nb >= SC_MAX_ACTIVE_INTERACTIONS) continue;
                    const sc_rule &pii = s.prules[(size_t)k];
                    if (!((p.type == pii.first_partner_type && tp.type == pii.second_partner_type) ||
                          (p.type == pii.second_partner_type && tp.type == pii.first_partner_type)) ||
                        pii.only_via_transition)
                        continue;
                    if (pii.group >= 0 && (group_active(p, pii.group) || group_active(tp, pii.group))) continue;
                    float oa, rpa;
                    alignment(p, tp, up, tup, delta, pii, &oa, &rpa);
                    if (oa > pii.orientation_alignment_threshold &&
                        fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold) &&
                        states_match(p, tp, pii) && bind_draw(s, pii, p.id, tp.id, step)) {
                        p.bonds[p.nb].type = pii.id;
                        p.bonds[p.nb].group = pii.group;
                        p.bonds[p.nb].partner_id = tp.id;
                        p.nb++;
                    }
                }
            });
        }
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// Complexify by deterministic pair claim (sc_config.pair_claim, an
// extension): every item with a free bond slot offers itself to each
// neighbour that some rule would bond it to, with the key (bits of
// |delta|^2 << 32 | its slot); every item keeps the lowest key offered to it,
// and two items bond when each holds the other's key, under the first rule
// that passes for the pair as seen from the lower slot.  At most one rule
// bond forms per item per step, on both sides.
int claim_rule(const scp_sim &s, const PP &a, const PP &b, sc_f3 delta, int step) {
    if (a.nb >= SC_MAX_ACTIVE_INTERACTIONS) return -1;
    int cs = 0, ce = 0;
    if (a.type >= 0 && (size_t)a.type * 2 + 1 < s.pidx.size()) { cs = s.pidx[a.type * 2]; ce = s.pidx[a.type * 2 + 1]; }
    const sc_f3 up = sc_rotate(sc_up(), a.rot), tup = sc_rotate(sc_up(), b.rot);
    for (int k = cs; k < ce; k++) {
        const sc_rule &pii = s.prules[(size_t)k];
        if (!((a.type == pii.first_partner_type && b.type == pii.second_partner_type) ||
              (a.type == pii.second_partner_type && b.type == pii.first_partner_type)) ||
            pii.only_via_transition)
            continue;
        if (pii.group >= 0 && (group_active(a, pii.group) || group_active(b, pii.group))) continue;
        float oa, rpa;
        alignment(a, b, up, tup, delta, pii, &oa, &rpa);
        if (oa > pii.orientation_alignment_threshold &&
            fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold) && states_match(a, b, pii) &&
            bind_draw(s, pii, a.id, b.id, step))
            return k;
    }
    return -1;
}

void complexify_claim(scp_sim &s, int step) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    std::vector<uint64_t> claim((size_t)std::max(n, 1), ~0ull);
    // offers, gathered per receiving item: the lowest key wins, so the order
    // in which they are made does not matter
    for (int i = 0; i < n; i++) {
        const PP &a = cur[i];
        if (!(a.flags & kActive) || a.nb >= SC_MAX_ACTIVE_INTERACTIONS) continue;
        s.scan(s.rangesP, a.pos, [&](int j) {
            if (j == i) return;
            const PP &b = cur[j];
            if (!(b.flags & kActive)) return;
            sc_f3 delta = s.img(b.pos, a.pos) - a.pos;
            if (outside_cube(delta, lim)) return;
            if (claim_rule(s, a, b, delta, step) < 0) return;
            const uint64_t key = ((uint64_t)sc_f2u(sc_normsq3(delta)) << 32) | (uint32_t)i;
            if (key < claim[(size_t)j]) claim[(size_t)j] = key;
        });
    }
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        const uint64_t key = claim[(size_t)i];
        if ((p.flags & kActive) && key != ~0ull) {
            const int j = (int)(uint32_t)key;
            if ((int)(uint32_t)claim[(size_t)j] == i) {
                const int lo = std::min(i, j), hi = std::max(i, j);
                const PP &a = cur[lo], &b = cur[hi];
                const int k = claim_rule(s, a, b, s.img(b.pos, a.pos) - a.pos, step);
                if (k >= 0 && p.nb < SC_MAX_ACTIVE_INTERACTIONS) {
                    const sc_rule &pii = s.prules[(size_t)k];
                    p.bonds[p.nb].type = pii.id;
                    p.bonds[p.nb].group = pii.group;
                    p.bonds[p.nb].partner_id = i == lo ? b.id : a.id;
                    p.nb++;
                }
            }
        }
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// ---- interactions.cuh:349-555 transitionInteractions -------------------------
void transition(scp_sim &s) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    const int step = s.step;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive) || p.nb < 1) { s.pn[i] = p; continue; }
        const sc_f3 up = sc_rotate(sc_up(), p.rot);
        int src = -1;
        sc_rule target = zero_rule();
        s.scan(s.rangesP, p.pos, [&](int j) {
            if (j == i) return;
            const PP &tp = cur[j];
            if (!(tp.flags & kActive)) return;
            sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
            if (outside_cube(delta, lim)) return;
            sc_f3 tup = sc_rotate(sc_up(), tp.rot);
            for (int k = 0; k < p.nb; k++) {
                sc_interaction it = p.bonds[k];
                if (it.type < 10) continue;
                if (it.partner_id != tp.id) continue;
                const sc_rule &pii = s.rule(it.type);
                if (!(pii.transition_to >= 0 || pii.break_after_transition)) continue;
                float oa, rpa;
                alignment(p, tp, up, tup, delta, pii, &oa, &rpa);
                bool aligned = pii.break_after_transition || !pii.wait_for_alignment ||
                               (oa > pii.orientation_alignment_threshold &&
                                fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold));
                if (!(aligned && (!pii.wait_for_state || states_match(p, tp, pii)))) continue;
                if (pii.transition_to >= 0) {
                    const sc_rule &tpii = s.rule(pii.transition_to);
                    if (tpii.group >= 0 && tpii.group != pii.group &&
                        (group_active(p, tpii.group) || group_active(tp, tpii.group)))
                        continue;
                    if (!tpii.set_state || !((p.type == tpii.first_partner_type && tpii.first_partner_state >= 0) ||
                                             (p.type == tpii.second_partner_type && tpii.second_partner_state >= 0))) {
                        p.bonds[k].type = tpii.id;
                        p.bonds[k].group = tpii.group;
                    } else {
                        src = k;
                        target = tpii;
                    }
                } else if (pii.break_after_transition) {
                    for (int l = k; l < p.nb - 1; l++) p.bonds[l] = p.bonds[l + 1];
                    p.nb--;
                    if (src > k) src--;
                    k--;
                }
            }
        });
        if (src >= 0) {
            p.bonds[src].type = target.id;
            p.bonds[src].group = target.group;
            if (target.set_state) {
                if (p.type == target.first_partner_type && target.first_partner_state >= 0) {
                    p.state = target.first_partner_state; p.lscs = step;
                }
                if (p.type == target.second_partner_type && target.second_partner_state >= 0) {
                    p.state = target.second_partner_state; p.lscs = step;
                }
            }
            if (target.polymerize >= 0) {
                const sc_rule &poly = s.rule(target.polymerize);
                if (poly.first_partner_type == p.type || poly.second_partner_type == p.type)
                    p.spoly = target.polymerize;
            }
        }
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// ---- interactions.cuh:558-740 polymerize (sequential, slot order) ----------
void polymerize(scp_sim &s) {
    const int n0 = s.nActive;
    std::vector<PP> &cur = s.p;
    for (int i = 0; i < n0; i++) {
        PP p = cur[i];
        if (!(p.flags & kActive) || p.spoly < 0) continue;
        const sc_rule poly = s.rule(p.spoly);
        int api = -1, pmi = -1;
        PP prev = make_particle(0, 0, 2.5f, SC_HYDROPHYLIC, sc_zero3(), sc_qid());
        for (int k = 0; k < p.nb; k++)
            if (p.bonds[k].group == poly.group) { api = k; break; }
        if (api >= 0) {
            int target = p.bonds[api].partner_id;
            s.scan(s.rangesP, p.pos, [&](int j) {
                if (j == i) return;
                const PP &tp = cur[j];
                if (!(tp.flags & kActive)) return;
                if (tp.id == target) { pmi = j; prev = tp; }
            });
        }
        bool first = poly.first_partner_type == p.type;
        int newType = first ? poly.second_partner_type : poly.first_partner_type;
        int newState = first ? poly.second_partner_state : poly.first_partner_state;
        if (newType >= 0) {
            sc_type_info ti;
            memset(&ti, 0, sizeof ti);
            if ((size_t)newType < s.types.size()) ti = s.types[(size_t)newType];
            int newIdx = ++s.lastActive;
            if (newIdx < s.N) {
                int newId = s.nextId++;
                sc_f3 rp = rule_pos(poly);
                sc_f4 ro = rule_ori(poly);
                sc_f3 npos = p.pos + sc_rotate(p.type < newType ? rp : -rp, p.rot);
                if (s.periodic) npos = sc_wrap3(npos, s.cfg.sim_size);
                PP np = make_particle(newId, newType, ti.radius, ti.hydrophobic, npos,
                                      sc_qmul(p.rot, p.type < newType ? ro : sc_qinv(ro)));
                if (newState >= 0) { np.state = (int8_t)newState; np.lscs = s.step; }
                np.bonds[np.nb] = {p.spoly, poly.group, p.id};
                np.nb++;
                if (pmi >= 0) {
                    for (int k = 0; k < prev.nb; k++) {
                        if (prev.bonds[k].group == poly.group) {
                            for (int l = k; l < prev.nb - 1; l++) prev.bonds[l] = prev.bonds[l + 1];
                            prev.nb--;
                            break;
                        }
                    }
                    prev.bonds[prev.nb] = {SC_INTERACTION_TYPE_CHAIN, SC_INTERACTION_GROUP_FORWARD, np.id};
                    prev.nb++;
                    cur[pmi] = prev;
                    np.bonds[np.nb] = {SC_INTERACTION_TYPE_CHAIN, SC_INTERACTION_GROUP_BACKWARD, prev.id};
                    np.nb++;
                    p.bonds[api].type = p.spoly;
                    p.bonds[api].partner_id = np.id;
                } else {
                    p.bonds[p.nb] = {p.spoly, poly.group, np.id};
                    p.nb++;
                }
                cur[newIdx] = np;
                s.nActive++;
            }
        } else {
            // End of the chain.  Without a previous monomer (pmi < 0) or an
            // active polymerisation bond (api < 0) the reference stores out
            // of bounds (interactions.cuh:728, 731-734); both stores are
            // skipped here.
            if (pmi >= 0) {
                for (int k = 0; k < prev.nb; k++) {
                    if (prev.bonds[k].group == poly.group) {
                        for (int l = k; l < prev.nb - 1; l++) prev.bonds[l] = prev.bonds[l + 1];
                        prev.nb--;
                        break;
                    }
                }
                cur[pmi] = prev;
            }
            if (api >= 0) {
                for (int l = api; l < p.nb - 1; l++) p.bonds[l] = p.bonds[l + 1];
                p.nb--;
            }
        }
        p.spoly = -1;
        cur[i] = p;
    }
}

// ---- interactions.cuh:743-822 propagateState ---------------------------------
// (main.cu:618-631 leaves its launch commented out: it runs here, after
// polymerize, only with sc_config.propagate_state.)  Each active particle
// below the post-polymerize count walks its 27 cells in order and, for every
// active neighbour inside the interaction cube that is the partner of one of
// its rule bonds (type >= 10) whose rule propagates state, takes the
// neighbour's state when the neighbour's last state change is later than its
// own (as updated so far).  Neighbours are read from the state before the pass.
void propagate_state(scp_sim &s) {
    const int n = s.nActive;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PP> &cur = s.p;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PP p = cur[i];
        if (p.flags & kActive) {
            s.scan(s.rangesP, p.pos, [&](int j) {
                if (j == i) return;
                const PP &tp = cur[j];
                if (!(tp.flags & kActive)) return;
                sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
                if (outside_cube(delta, lim)) return;
                // (a count past the 8 slots, which polymerize can leave, reads
                // the 8 slots: the reference would read past the array)
                for (int k = 0; k < std::min(p.nb, SC_MAX_ACTIVE_INTERACTIONS); k++) {
                    const sc_interaction &it = p.bonds[k];
                    if (it.type < 10 || it.partner_id != tp.id) continue;
                    if (!s.rule(it.type).propagate_state) continue;
                    if (tp.lscs > p.lscs) {
                        p.lscs = tp.lscs;
                        p.state = tp.state;
                    }
                }
            });
        }
        s.pn[i] = p;
    }
    clear_tail(s.pn, n);
    s.p.swap(s.pn);
}

// ---- metabolites.cuh:352-431 diffuseMetabolites ------------------------------
void diffuse(scp_sim &s) {
    const int n = s.nActiveM;
    const float lim = s.cfg.max_diffusion_distance;
    const int S = s.S;
    const std::vector<PM> &cur = s.m;
    const float thr = 0.001f;  // only used through the double comparison below
    (void)thr;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PM p = cur[i];
        if (!(p.flags & kActive)) { s.mn[i] = p; continue; }
        float dm[SC_AOS_NUM_METABOLITES] = {0};
        s.scan(s.rangesM, p.pos, [&](int j) {
            if (j == i) return;
            const PM &tp = cur[j];
            if (!(tp.flags & kActive)) return;
            sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
            if (outside_cube(delta, lim)) return;
            float dist = sc_norm3(delta);
            if (dist <= lim) {
                for (int k = 0; k < S; k++) {
                    float diff = tp.m[k] - p.m[k];
                    if ((double)fabsf(diff) > 0.001) dm[k] += diff * 0.1f;
                }
            }
        });
        for (int k = 0; k < S; k++) p.m[k] += dm[k];
        s.mn[i] = p;
    }
    clear_tail(s.mn, n);
    s.m.swap(s.mn);
}

// ---- metabolites.cuh:18-88 removeInterferingMetabolicParticles --------------
void remove_interfering(scp_sim &s) {
    const int n = s.nActiveM;
    const float lim = s.cfg.max_interaction_distance;
    const std::vector<PM> &cur = s.m;
    const std::vector<PP> &parts = s.p;
    SC_OMP_FOR
    for (int i = 0; i < n; i++) {
        PM p = cur[i];
        if (!(p.flags & kActive)) { s.mn[i] = p; continue; }
        s.scan(s.rangesP, p.pos, [&](int j) {
            const PP &tp = parts[j];
            if (!(tp.flags & kActive) || tp.type != SC_PARTICLE_TYPE_LIPID) return;
            sc_f3 delta = s.img(tp.pos, p.pos) - p.pos;
            if (outside_cube(delta, lim)) return;
            float dist = sc_norm3(delta);
            float interf = (float)((double)(p.radius + tp.radius) + 0.001);
            if (dist <= interf) p.flags = p.flags & ~kActive;
        });
        s.mn[i] = p;
    }
    clear_tail(s.mn, n);
    s.m.swap(s.mn);
}

template <class T, class R>
void reduce_one(const T &p, R &r) {
    r.id = p.id;
    r.type = p.type;
    r.flags = p.flags | (((int)p.state & 0x0000000F) << 16);
    r.radius = sc_f2h(p.radius);
    r.pos[0] = sc_f2h(p.pos.x); r.pos[1] = sc_f2h(p.pos.y); r.pos[2] = sc_f2h(p.pos.z);
    r.rot[0] = sc_f2h(p.rot.x); r.rot[1] = sc_f2h(p.rot.y); r.rot[2] = sc_f2h(p.rot.z); r.rot[3] = sc_f2h(p.rot.w);
    r.debug_vector[0] = sc_f2h(p.dbg.x); r.debug_vector[1] = sc_f2h(p.dbg.y);
    r.debug_vector[2] = sc_f2h(p.dbg.z); r.debug_vector[3] = sc_f2h(p.dbg.w);
}

}  // namespace

extern "C" {

#if !defined(SC_PORT_FP64)
// ---- scmath.h entry points for the CPU tests ---------------------------------
// fn: 0 sin, 1 cos, 2 acos, 3 log, 4 exp, 5 pow(x, y)
void scp_math_eval(int fn, const float *x, const float *y, float *out, int n) {
    for (int i = 0; i < n; i++) {
        switch (fn) {
            case 0: out[i] = sc_sinf(x[i]); break;
            case 1: out[i] = sc_cosf(x[i]); break;
            case 2: out[i] = sc_acosf(x[i]); break;
            case 3: out[i] = sc_logf(x[i]); break;
            case 4: out[i] = sc_expf(x[i]); break;
            default: out[i] = sc_powf(x[i], y[i]); break;
        }
    }
}
void scp_philox(const uint32_t *ctr, uint32_t k0, uint32_t k1, uint32_t *out) {
    sc_u4 c = {ctr[0], ctr[1], ctr[2], ctr[3]};
    sc_u4 o = sc_philox4x32_10(c, k0, k1);
    out[0] = o.x; out[1] = o.y; out[2] = o.z; out[3] = o.w;
}
// The device scene generator's records (sc_gen.h) built on the host.
int scp_generate_uniform(int32_t n, int32_t nm, const int32_t *kinds, const float *fractions, int32_t nkinds,
                         const sc_type_info *types, int32_t ntypes, float box, int32_t species, uint64_t seed,
                         sc_particle *p, sc_metabolic_particle *m) {
    sc_gen_mix mix;
    if (n > 0 && sc_gen_make_mix(&mix, kinds, fractions, nkinds, types, ntypes)) return -1;
    for (int32_t i = 0; i < n; i++) sc_gen_particle(&p[i], i, box, &mix, seed);
    for (int32_t j = 0; j < nm; j++)
        sc_gen_metabolic(&m[j], j, box, species, types[SC_PARTICLE_TYPE_METABOLIC].radius,
                         types[SC_PARTICLE_TYPE_METABOLIC].hydrophobic, seed);
    return 0;
}

// The structured scene generator's records (sc_gen.h) built on the host:
// returns the particle count, or -1 for an invalid group list.
int64_t scp_generate_scene(const sc_scene_group *groups, int32_t ng, int32_t nm, const sc_type_info *types,
                           int32_t ntypes, float box, int32_t species, uint64_t seed, sc_particle *p,
                           sc_metabolic_particle *m) {
    std::vector<sc_gen_group> gg((size_t)(ng > 0 ? ng : 1));
    const char *why = "";
    const int64_t n = sc_gen_prepare(groups, ng, types, ntypes, gg.data(), &why);
    if (n < 0) return -1;
    if (!p) return n;  // size query
    for (int32_t g = 0; g < ng; g++) {
        const sc_gen_group &G = gg[(size_t)g];
        const int per = (G.kind == SC_SCENE_COMPLEXES || G.kind == SC_SCENE_WRAPPED_CHAINS) ? G.unit : 1;
        for (int32_t u = 0; u < G.count; u++) sc_gen_unit(&p[G.first + (int64_t)u * per], &G, u, box, seed);
    }
    for (int32_t j = 0; j < nm; j++)
        sc_gen_metabolic(&m[j], j, box, species, types[SC_PARTICLE_TYPE_METABOLIC].radius,
                         types[SC_PARTICLE_TYPE_METABOLIC].hydrophobic, seed);
    return n;
}

void scp_f2h(const float *x, uint16_t *out, int n) {
    for (int i = 0; i < n; i++) out[i] = sc_f2h(x[i]);
}
void scp_draws(uint64_t seed, uint32_t stream, uint32_t id0, int n, uint32_t step, uint32_t d, int normal,
               float *out) {
    for (int i = 0; i < n; i++)
        out[i] = normal ? sc_normal(seed, stream, id0 + (uint32_t)i, step, d)
                        : sc_uniform(seed, stream, id0 + (uint32_t)i, step, d);
}
// 1 where the single-precision form of a double comparison disagrees with it.
// kind 0: lipid range (dist, s); kind 1: diffusion threshold (x);
// kind 2: metabolic collision distance (rp, rt); kind 3: polar attraction (L);
// kind 4: Brownian step length (x, radius); kind 5: rotation weight (rn, radius).
// Values are compared as bit patterns.
static bool same_bits(float x, float y) { return sc_f2u(x) == sc_f2u(y) || (x != x && y != y); }
void scp_compare_forms(int kind, const float *a, const float *b, uint8_t *bad, int n) {
    for (int i = 0; i < n; i++) {
        if (kind == 0) {
            bool exact = (double)a[i] <= (double)b[i] + 0.8 * (double)b[i] * 0.5;
            bad[i] = sc_within_lipid_range(a[i], b[i]) != exact;
        } else if (kind == 2) {
            bad[i] = !same_bits(sc_coll_dist(a[i], b[i]), metab_collision_dist(a[i], b[i]));
        } else if (kind == 4) {
            bad[i] = !same_bits(sc_noise_mag(a[i], b[i]),
                                (float)((double)a[i] / fmax((double)b[i] / 2.5, 1.0)));
        } else if (kind == 5) {
            bad[i] = !same_bits(sc_rot_noise(a[i], b[i]), (float)((double)a[i] / ((double)b[i] / 2.5)));
        } else if (kind == 3) {
            float L = a[i];
            bad[i] = !same_bits(sc_polar_attr(L), (float)(fmin(fmax((double)L, 1e-6), (double)2.0f) / (double)2.0f));
        } else {
            bool exact = (double)fabsf(a[i]) > 0.001;
            bad[i] = sc_diffuse_exceeds(a[i]) != exact;
        }
    }
}

#endif  // !SC_PORT_FP64

void scp_set_threads(int n) {
#if defined(_OPENMP)
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int scp_max_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

scp_sim *scp_create(const sc_config *cfg, const sc_type_info *types, int n_types, const sc_rule *rules, int n_rules) {
    if (!cfg || cfg->num_particles < 0 || cfg->num_metabolic_particles < 0) return nullptr;
    if (cfg->num_metabolites < 1 || cfg->num_metabolites > SC_AOS_NUM_METABOLITES) return nullptr;
    scp_sim *s = new scp_sim();
    s->cfg = *cfg;
    s->S = cfg->num_metabolites;
    // config.cuh:65-74
    int ng = (int)ceilf(cfg->sim_size / cfg->grid_cell_size);
    int bits = 1, p2 = 2;
    while (p2 < ng) { p2 *= 2; bits++; }
    s->ngrid = p2;
    s->nbits = bits;
    s->periodic = cfg->periodic != 0;
    s->nUsed = ng;
    s->cellSize = cfg->grid_cell_size;
    if (s->periodic) {
        sc_single width = 0;
        s->nUsed = sc_periodic_cells(cfg->sim_size, cfg->grid_cell_size, &width);
        s->cellSize = width;
    }
    if (s->periodic && s->nUsed < 3) { delete s; return nullptr; }
    s->cells = (size_t)p2 * p2 * p2;
    s->N = cfg->num_particles;
    s->Nm = cfg->num_metabolic_particles;
    s->p.assign((size_t)s->N, PP());
    s->pn.assign((size_t)s->N, PP());
    s->m.assign((size_t)s->Nm, PM());
    s->mn.assign((size_t)s->Nm, PM());
    if (s->N) memset((void *)s->p.data(), 0, s->p.size() * sizeof(PP));
    if (s->Nm) memset((void *)s->m.data(), 0, s->m.size() * sizeof(PM));
    s->rangesP.assign(s->cells * 2, 0);
    s->rangesM.assign(s->cells * 2, 0);
    s->types.assign(types, types + std::max(n_types, 0));
    int maxId = 0;
    for (int i = 0; i < n_rules; i++) maxId = std::max(maxId, rules[i].id);
    s->flat.assign((size_t)maxId + 1, zero_rule());
    std::vector<char> seen((size_t)maxId + 1, 0);
    for (int i = 0; i < n_rules; i++) {
        int id = rules[i].id;
        if (id < 0 || seen[(size_t)id]) continue;
        seen[(size_t)id] = 1;
        s->flat[(size_t)id] = rules[i];
        if (!cfg->rule_probabilities) {  // padding in the reference's records
            s->flat[(size_t)id].use_probability = 0;
            s->flat[(size_t)id].probability = 0.0f;
        }
    }
    // partner index (interactions.cuh:79-145), rules in ascending id per type
    s->pidx.assign(((size_t)maxId + 1) * 2, 0);
    std::map<int, std::vector<int>> byType;
    for (int id = 0; id <= maxId; id++) {
        if (!seen[(size_t)id]) continue;
        const sc_rule &r = s->flat[(size_t)id];
        if (r.first_partner_type >= 0) byType[r.first_partner_type].push_back(id);
        if (r.second_partner_type >= 0) byType[r.second_partner_type].push_back(id);
    }
    for (auto &kv : byType) {
        int start = (int)s->prules.size();
        for (int id : kv.second) s->prules.push_back(s->flat[(size_t)id]);
        if ((size_t)kv.first * 2 + 1 < s->pidx.size()) {
            s->pidx[(size_t)kv.first * 2] = start;
            s->pidx[(size_t)kv.first * 2 + 1] = (int)s->prules.size();
        }
    }
    return s;
}

void scp_destroy(scp_sim *s) { delete s; }

int scp_load_state(scp_sim *s, const sc_particle *p, int n, const sc_metabolic_particle *m, int nm, int step,
                   int next_id) {
    if (n < 0 || nm < 0 || n > s->N || nm > s->Nm) return SC_E_INVALID;
    if (s->N) memset((void *)s->p.data(), 0, s->p.size() * sizeof(PP));
    if (s->Nm) memset((void *)s->m.data(), 0, s->m.size() * sizeof(PM));
    if (n) put_particles(s->p.data(), p, n);
    if (nm) put_metabolic(s->m.data(), m, nm);
    s->nActive = n; s->lastActive = n - 1; s->nextId = next_id; s->nActiveM = nm; s->step = step;
    return SC_OK;
}

int scp_run_phase(scp_sim *s, int phase, int arg) {
    switch (phase) {
        case SC_PHASE_SORT_PARTICLES:
            sort_items(*s, s->p, s->pn, s->keyP, s->permP, s->rangesP, s->N);
            s->lastActive = s->nActive - 1;
            break;
        case SC_PHASE_SORT_METABOLIC:
            sort_items(*s, s->m, s->mn, s->keyM, s->permM, s->rangesM, s->Nm);
            break;
        case SC_PHASE_MOVE_BROWNIAN:
            move_items(s->p, s->pn, s->nActive);
            brownian(*s, s->p, s->nActive, s->cfg.movement_noise_scale, SC_STREAM_P_UNIFORM, SC_STREAM_P_NORMAL);
            break;
        case SC_PHASE_MOVE_BROWNIAN_METAB:
            move_items(s->m, s->mn, s->nActiveM);
            brownian(*s, s->m, s->nActiveM, s->cfg.metabolite_movement_noise_scale, SC_STREAM_M_UNIFORM,
                     SC_STREAM_M_NORMAL);
            break;
        case SC_PHASE_COORDINATE_NOISE:
            coordinate_noise(*s, (float)arg / s->cfg.noise_coordination_steps);
            break;
        case SC_PHASE_APPLY_NOISE:
            apply_noise(s->p, s->nActive);
            apply_noise(s->m, s->nActiveM);
            break;
        case SC_PHASE_RELAX: relax(*s); break;
        case SC_PHASE_RELAX_METAB: relax_metab(*s); break;
        case SC_PHASE_RELAX_PARTNERS: relax_partners(*s); break;
        case SC_PHASE_APPLY_VELOCITIES:
            apply_velocities(*s, s->p, s->nActive, 0.45f);
            apply_velocities(*s, s->m, s->nActiveM, 0.45f);
            break;
        case SC_PHASE_COMPLEXIFY: complexify(*s, arg == -1 ? -1 : s->step); break;
        case SC_PHASE_TRANSITION: transition(*s); break;
        case SC_PHASE_POLYMERIZE: polymerize(*s); break;
        case SC_PHASE_DIFFUSE: diffuse(*s); break;
        case SC_PHASE_REMOVE_INTERFERING: remove_interfering(*s); break;
        case SC_PHASE_END_STEP: s->step++; break;
        case SC_PHASE_PROPAGATE_STATE: propagate_state(*s); break;
        default: return SC_E_INVALID;
    }
    return SC_OK;
}

int scp_prepare(scp_sim *s) {
    scp_run_phase(s, SC_PHASE_SORT_PARTICLES, 0);
    scp_run_phase(s, SC_PHASE_SORT_METABOLIC, 0);
    scp_run_phase(s, SC_PHASE_REMOVE_INTERFERING, 0);
    scp_run_phase(s, SC_PHASE_COMPLEXIFY, -1);
    return SC_OK;
}

int scp_step(scp_sim *s, int n_steps) {
    for (int k = 0; k < n_steps; k++) {
        scp_run_phase(s, SC_PHASE_SORT_PARTICLES, 0);
        scp_run_phase(s, SC_PHASE_SORT_METABOLIC, 0);
        scp_run_phase(s, SC_PHASE_MOVE_BROWNIAN, 0);
        scp_run_phase(s, SC_PHASE_MOVE_BROWNIAN_METAB, 0);
        for (int j = 0; j < s->cfg.noise_coordination_steps; j++) scp_run_phase(s, SC_PHASE_COORDINATE_NOISE, j);
        scp_run_phase(s, SC_PHASE_APPLY_NOISE, 0);
        for (int j = 0; j < s->cfg.relaxation_steps; j++) {
            scp_run_phase(s, SC_PHASE_RELAX, j);
            if (j % 2 == 0) {
                scp_run_phase(s, SC_PHASE_RELAX_METAB, j);
                scp_run_phase(s, SC_PHASE_RELAX_PARTNERS, j);
            }
        }
        scp_run_phase(s, SC_PHASE_APPLY_VELOCITIES, 0);
        scp_run_phase(s, SC_PHASE_COMPLEXIFY, s->step);
        scp_run_phase(s, SC_PHASE_TRANSITION, 0);
        scp_run_phase(s, SC_PHASE_POLYMERIZE, 0);
        if (s->cfg.propagate_state) scp_run_phase(s, SC_PHASE_PROPAGATE_STATE, 0);
        for (int j = 0; j < s->cfg.metabolite_diffusion_steps; j++) scp_run_phase(s, SC_PHASE_DIFFUSE, j);
        scp_run_phase(s, SC_PHASE_END_STEP, 0);
    }
    return SC_OK;
}

int scp_export_state(scp_sim *s, sc_particle *p, sc_metabolic_particle *m) {
    if (p && s->N) get_particles(p, s->p.data(), s->N);
    if (m && s->Nm) get_metabolic(m, s->m.data(), s->Nm);
    return SC_OK;
}

int scp_export_grid(scp_sim *s, int which, uint32_t *ranges, uint32_t *perm) {
    const std::vector<uint32_t> &r = which ? s->rangesM : s->rangesP;
    const std::vector<uint32_t> &q = which ? s->permM : s->permP;
    if (ranges) memcpy(ranges, r.data(), r.size() * 4);
    if (perm && !q.empty()) memcpy(perm, q.data(), q.size() * 4);
    return SC_OK;
}

int scp_get_counters(scp_sim *s, sc_counters *c) {
    memset(c, 0, sizeof *c);
    c->n_active_particles = s->nActive;
    c->n_active_metabolic_particles = s->nActiveM;
    c->next_particle_id = s->nextId;
    c->step = s->step;
    return SC_OK;
}

int scp_reduce_frame(scp_sim *s, sc_reduced_particle *rp, sc_reduced_metabolic_particle *rm) {
    if (rp) {
        memset(rp, 0, (size_t)s->N * sizeof *rp);
        for (int i = 0; i < s->nActive && i < s->N; i++) reduce_one(s->p[i], rp[i]);
    }
    if (rm) {
        memset(rm, 0, (size_t)s->Nm * sizeof *rm);
        for (int i = 0; i < s->nActiveM && i < s->Nm; i++) {
            reduce_one(s->m[i], rm[i].p);
            for (int k = 0; k < SC_REDUCED_NUM_METABOLITES; k++) rm[i].metabolites[k] = sc_f2h(s->m[i].m[k]);
        }
    }
    return SC_OK;
}

}  // extern "C"
