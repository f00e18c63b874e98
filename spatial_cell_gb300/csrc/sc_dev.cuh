// sc_dev.cuh -- device-side layout and helpers of the sm_103a step.
//
// State lives in HBM as structure-of-arrays (one float4 / int4 per item per
// field) instead of the reference's 256 / 304-byte structs (types.cuh:173-242),
// so every kernel moves only the fields it touches, 16 bytes at a time:
//
//   particles   pos      float4  x y z | radius
//               vel      float4  x y z | -        (ping-pong inside a step)
//               rot      float4  quaternion        (ping-pong in relax)
//               angvel   float4                    (ping-pong)
//               posnoise float4  x y z | -         (ping-pong in coordinateNoise)
//               angnoise float4                    (ping-pong in coordinateNoise)
//               info     int4    id | type | flags | state(8) hydrophobic(8)
//               dbg      float4  debugVector
//               lscs, spoly, nb  int               lastStateChangeStep,
//                                                  scheduledPolymerization,
//                                                  nActiveInteractions
//               bonds    int[24] interactions[8] {type, group, partnerId}
//   metabolic   pos vel rot angvel posnoise angnoise info dbg as above,
//               met float[SP] per item (S species padded to a multiple of 4),
//               orig int: load slot of the item, indexing the fields no step
//               kernel reads or writes (lscs, spoly, bonds), kept in load order.
//
// Every sort gathers all fields into the other buffer of each pair, so the
// sorted order of every array is the sorted order of the keys, as in the
// reference where CUB moves the whole struct (grid.cuh:91-103).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "scmath.h"
#include "spatialcell.h"

#define SC_THREADS 256
#define SC_ACTIVE SC_PARTICLE_FLAG_ACTIVE

// Pair lists.  Between a sort and applyVelocities no position, flag, type,
// radius or interaction changes, so the pairs that contribute to
// coordinateNoise / relax / relaxMetabolicParticles /
// relaxMetabolicParticlePartners are fixed for all of their sub-iterations
// (16 / 32 / 16 / 16 launches); likewise the diffusion pairs between
// applyVelocities and the next sort (8 launches).  Each list holds, per item
// and in the reference's visiting order, the candidate slots that pass every
// position-only test of the kernel, with the branch the pair takes.  Entries
// are tiled by warps of 32 items: entry k of item i is at
// ((i / 32) * K + k) * 32 + i % 32, so the 32 threads of a warp read one
// 128-byte line per k and all K entries of a warp sit in one K*128-byte block
// (one page, where a k-major layout would put each k of an item in a different
// page).  An item with more pairs than the list holds is marked by a count
// above the capacity and its kernels scan its neighbourhood instead.
#define SC_LIST_PP 128  // particle-particle: rule/chain/test bonds, polar pairs, collisions (dense
                        // lipid membranes list ~100)
#define SC_LIST_M 160   // metabolic: colliding metabolic particles and lipids (beside a dense
                        // membrane ~110)
#define SC_LIST_LM 48   // lipid <- metabolic collisions
#define SC_LIST_D 96    // metabolic diffusion partners
// The diffusion list's buffer holds the count-ordered diffusion list and,
// after it, the diffusion list's build scratch; the whole buffer is also the
// build scratch of the metabolic list (whose pool is sized by demand).
#define SC_LIST_DBUF (SC_LIST_M > 2 * SC_LIST_D ? SC_LIST_M : 2 * SC_LIST_D)
#define SC_PP_POLAR 0x80000000u
#define SC_PP_PARTNER 0x40000000u
#define SC_PP_COLLIDE 0x20000000u
#define SC_PP_INDEX 0x1FFFFFFFu
#define SC_M_FROM_P 0x80000000u
#define SC_M_INDEX 0x7FFFFFFFu

__host__ __device__ __forceinline__ size_t sc_list_at(int K, int i, int k) {
    return ((size_t)(i >> 5) * (size_t)K + (size_t)k) * 32 + (size_t)(i & 31);
}
__host__ __device__ __forceinline__ size_t sc_list_words(int K, int cap) { return (size_t)((cap + 31) / 32) * 32 * K; }

// Device-side error codes (sticky, first one wins).
#define SC_DERR_LOOKBACK_TIMEOUT 1
#define SC_DERR_POLY_OVERFLOW 2

struct ScCounters {
    int nActive;      // nActiveParticles (main.cu:244), bound of every particle kernel
    int lastActive;   // lastActiveParticle (main.cu:245)
    int nextId;       // nextParticleId (main.cu:246)
    int nActiveM;     // nActiveMetabolicParticles (main.cu:253)
    int error;        // first device-side error code
    int polyCount;    // scheduled polymerisations listed this step (k_poly_offsets)
    int polyCreates;  // of those, the ones whose rule creates a monomer
    int polyConflict; // 1: two listed items touch the same particle (k_poly_plan)
    int step;         // the step loop counter (main.cu:347)
    int tileCounter[4];
    int ppClassCount[4];  // items per relax work class (k_build_pp)
    int ovfPP, ovfM;      // items whose particle / metabolic list overflowed (k_build_pp, k_build_m)
    int _pad;
    unsigned long long poolM;   // entries the metabolic list blocks asked of their pool (k_build_m)
    unsigned long long poolLM;  // the same for the lipid-metabolic lists (k_build_lm)
    int workCount;              // items in the particle work list (k_complexify_select)
    int ovfD;                     // items whose diffusion list overflowed (k_build_d)
    unsigned long long poolOvfM;  // entries the overflowed metabolic items asked of their pool (k_build_m_ovf)
    unsigned long long poolOvfD;  // the same for the diffusion lists (k_build_d_ovf)
};

// Relax work classes: 0 bonded items, 1 items with polar (lipid) pairs and no
// bonds, 2 the rest.  Each class has its own kernel, so a warp's items take
// the same branches.
#define SC_RELAX_CLASSES 3
// Bond match count of a bonded item (low bits) and its in-order flag (a
// test bond: relaxed by the in-order scan).
#define SC_MATCH_COUNT 0xff
#define SC_MATCH_INORDER 0x100

// The geometry of one replica of a batched sim (sc_create_batch): its box,
// its cells, where its cells start in the batch's key space, its noise key.
struct ScRep {
    float simSize, cell;
    int ngrid, bits, nUsed;
    uint32_t keyBase;
    uint64_t seed;
};

struct ScParams {
    float simSize, maxInt, maxDiff, cell;
    int ngrid, bits;
    uint32_t cells;           // cells of the key space (all replicas of a batch)
    uint32_t keyBase;         // first key of this item's replica (0 outside batches)
    int keyBits;              // key bits the sort orders (3 * bits + 1 outside batches)
    int nRep;                 // replicas of a batched sim (1 otherwise)
    const ScRep *reps;        // their geometry (batched sims)
    float moveNoise, rotNoise, metabNoise, velDecay, angDecay;
    int S, SP;
    int N, Nm;
    int coordSteps;
    uint64_t seed;
    const sc_rule *flat;      // id-indexed rules (flattenComplexificationInfo) + one zero rule
    int nFlat;
    const int *pidx;          // partner index [2 * type] -> [start, end)
    int nPidx;
    const sc_rule *prules;    // partner-mapped rules
    const sc_type_info *types;
    int nTypes;
    int listLimit;            // effective pair-list capacity (<= each list's size; smaller only in tests)
    int periodic;             // periodic box extension (sc_config.periodic)
    int walls;                // walled box: 0 clamp (reference), 1 reflect (sc_config.walls)
    int pairClaim;            // complexify by deterministic pair claim (sc_config.pair_claim)
    int metabLean;            // metabolic pair pool of 4-byte entries, geometry evaluated per sub-iteration
                              // (sc_config.metabolic_pairs 0); else 16-byte entries with it frozen (1, default)
    int nUsed;                // cells per axis the box spans, ceil(simSize / cell)
    int binned;               // SC_BINNED_*: sets whose positions are those their cells were sorted by
    int tileCapM, tileCapP;   // tile capacities (slots) of the metabolic sweeps; 0: tiles off
    // Candidate tests that need no record load: after a metabolic sort every
    // binned metabolic item is active (inactive ones sort past the cells)
    // until removeInterferingMetabolicParticles; after a particle sort
    // lipidP[slot] says "active lipid" (types and particle flags do not
    // change between sorts).
    int mAllActive;
    int lipidValid;
    const uint8_t *lipidP;
};

// Whether sorted particle j is an active lipid.
__device__ __forceinline__ bool active_lipid(const ScParams &P, const int4 *__restrict__ pinfo, int j) {
    if (P.lipidValid) return P.lipidP[j] != 0;
    const int4 tin = pinfo[j];
    return (tin.z & SC_ACTIVE) && tin.y == SC_PARTICLE_TYPE_LIPID;
}
// Whether sorted metabolic item j is active.
__device__ __forceinline__ bool active_m(const ScParams &P, const int4 *__restrict__ minfo, int j) {
    return P.mAllActive || (minfo[j].z & SC_ACTIVE);
}
#define SC_BINNED_P 1
#define SC_BINNED_M 2

// Cells per axis the cell index clamps to: the power-of-two grid of
// config.cuh:65-74, or in a periodic box the cells the box spans.
__host__ __device__ __forceinline__ int cell_limit(const ScParams &P) { return P.periodic ? P.nUsed : P.ngrid; }

// A neighbour's position as seen from an item at p: itself, or in a periodic
// box its nearest image.  When the neighbours' sets (need, SC_BINNED_*) still
// sit in the cells they were sorted into, neighbours from the 27 cells around
// p are less than 2.5 cells away per axis; if p's cell is not on a face of a
// periodic box at least 5 cells wide, that is less than half the box and
// every neighbour is its own nearest image, so the test is made once per item.
struct Imager {
    bool wrap;
    float L;
    sc_f3 p;
    __device__ __forceinline__ Imager(const ScParams &P, sc_f3 pos, int need) : wrap(false), L(P.simSize), p(pos) {
        if (P.periodic && (P.binned & need) != need) {
            wrap = true;
        } else if (P.periodic) {
            int n = P.nUsed;
            int cx = (int)sc_grid_idx(pos.x, P.cell, n), cy = (int)sc_grid_idx(pos.y, P.cell, n),
                cz = (int)sc_grid_idx(pos.z, P.cell, n);
            wrap = !(P.simSize >= 5.0f * P.cell) || cx == 0 || cy == 0 || cz == 0 || cx == n - 1 || cy == n - 1 ||
                   cz == n - 1;
        }
    }
    __device__ __forceinline__ sc_f3 operator()(sc_f3 t) const { return wrap ? sc_image3(t, p, L) : t; }
};

__device__ __forceinline__ sc_f4 ld4(const float4 *p, int i) {
    float4 v = p[i];
    return sc_make_f4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ sc_f3 ld3(const float4 *p, int i) {
    float4 v = p[i];
    return sc_make_f3(v.x, v.y, v.z);
}
__device__ __forceinline__ void st4(float4 *p, int i, sc_f4 v) { p[i] = make_float4(v.x, v.y, v.z, v.w); }

// A 32-byte row (two float4, 32-byte aligned) in one 256-bit access
// (ld/st .v8 on the global space, sm_100 and later): a warp's scattered rows
// then cost one L1 wavefront per row instead of two.  The load is for
// buffers no thread writes during the kernel.
__device__ __forceinline__ void ld_row8(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void st_row8(float4 *p, float4 a, float4 b) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}
__device__ __forceinline__ void st3(float4 *p, int i, sc_f3 v, float w) { p[i] = make_float4(v.x, v.y, v.z, w); }

__device__ __forceinline__ int info_state(int w) { return (int)(int8_t)(w & 0xff); }
__device__ __forceinline__ int info_hydro(int w) { return (int)(int8_t)((w >> 8) & 0xff); }
__device__ __forceinline__ int info_pack(int state, int hydro) { return (state & 0xff) | ((hydro & 0xff) << 8); }

// flat[] holds nFlat id-indexed rules plus one zero rule at [nFlat]: ids
// without a rule read as all-zero, as the reference's memset table does.
__device__ __forceinline__ const sc_rule &rule_at(const ScParams &P, int id) {
    return P.flat[(id >= 0 && id < P.nFlat) ? id : P.nFlat];
}
__device__ __forceinline__ sc_f4 rule_ori(const sc_rule &r) {
    return sc_make_f4(r.relative_orientation[0], r.relative_orientation[1], r.relative_orientation[2],
                      r.relative_orientation[3]);
}
__device__ __forceinline__ sc_f3 rule_pos(const sc_rule &r) {
    return sc_make_f3(r.relative_position[0], r.relative_position[1], r.relative_position[2]);
}

__device__ __forceinline__ bool outside_cube(sc_f3 d, float lim) {
    return fabsf(d.x) > lim || fabsf(d.y) > lim || fabsf(d.z) > lim;
}

__device__ __forceinline__ uint32_t cell_key(const ScParams &P, uint32_t gx, uint32_t gy, uint32_t gz) {
    return P.keyBase + ((gx << (2 * P.bits)) | (gy << P.bits) | gz);
}

// Batched sims: every item carries its replica in the bits of its info
// record's w word above the hydrophobicity byte.  A kernel of a batch works
// on one item at a time with that replica's geometry (its neighbours are in
// the same replica's cells); outside batches P is used as given.
__device__ __forceinline__ int item_rep(int infoW) { return (int)((unsigned)infoW >> 8); }
template <bool BATCH>
__device__ __forceinline__ void rep_apply(ScParams &P, int infoW) {
    if (!BATCH) return;
    const int r = min(item_rep(infoW), P.nRep - 1);
    const ScRep g = P.reps[r];
    P.simSize = g.simSize;
    P.cell = g.cell;
    P.ngrid = g.ngrid;
    P.bits = g.bits;
    P.nUsed = g.nUsed;
    P.keyBase = g.keyBase;
    P.seed = g.seed;
}

// Visits the reference's 27-cell neighbourhood of pos (grid.cuh:13-25 and the
// loop of e.g. dynamics.cuh:445-451): cells clamped at the box edge, in gx, gy,
// gz order, slots ascending inside a cell.  Keys of the cells (gx, gy, z0..z1)
// are consecutive, so with the exclusive cell-start table (cellStart[c] =
// first sorted slot with key >= c) that run of cells is one slot range, and
// the visiting order is exactly the reference's.
// Offsets (-1..1 per axis) of the neighbour cells a scan visits.  All 27 by
// default; reach() drops a neighbour layer when no item in it can pass the
// interaction cube |delta| <= lim on that axis, which every caller tests
// before anything else, so the visits that remain are the reference's, in its
// order, and the results are unchanged.  The bound needs the neighbours to
// sit in the cells they were sorted into (P.binned covers `need`), lim at
// most the cell size, and a periodic box of at least 5 cells (no nearest image
// crosses back into the cube).  Candidates of cell c - 1 lie below c * cell
// and those of cell c + 1 at or above (c + 1) * cell (or at the box size
// past the top periodic cell), up to the rounding of the cell index; the
// margin covers that and the rounding of delta.
struct Reach {
    int xl = -1, xh = 1, yl = -1, yh = 1, zl = -1, zh = 1;
};
__device__ __forceinline__ void reach_axis(const ScParams &P, float p, int c, int n, float lim, int &lo, int &hi) {
    const float m = lim + 1e-3f + 4e-6f * (fabsf(p) + P.cell * (float)(c + 1));
    lo = (p - (float)c * P.cell > m) ? 0 : -1;
    const float upper = (P.periodic && c == n - 1) ? P.simSize : (float)(c + 1) * P.cell;
    hi = (upper - p > m) ? 0 : 1;
}
__device__ __forceinline__ Reach reach(const ScParams &P, sc_f3 pos, float lim, int need) {
    Reach r;
    if ((P.binned & need) != need || !(lim <= P.cell) || (P.periodic && !(P.simSize >= 5.0f * P.cell))) return r;
    const int n = cell_limit(P);
    reach_axis(P, pos.x, (int)sc_grid_idx(pos.x, P.cell, n), n, lim, r.xl, r.xh);
    reach_axis(P, pos.y, (int)sc_grid_idx(pos.y, P.cell, n), n, lim, r.yl, r.yh);
    reach_axis(P, pos.z, (int)sc_grid_idx(pos.z, P.cell, n), n, lim, r.zl, r.zh);
    return r;
}

// A neighbour cell index c + o (c in [0, n), o in -1..1) taken around the
// periodic box: ((c + o + n) mod n) without the integer division.
__device__ __forceinline__ uint32_t wrap_cell(int v, int n) {
    return (uint32_t)(v < 0 ? v + n : (v >= n ? v - n : v));
}

template <class F>
__device__ __forceinline__ void scan27(const ScParams &P, const uint32_t *__restrict__ cellStart, sc_f3 pos,
                                       const Reach &R, F &&f) {
    int n = cell_limit(P);
    int cx = (int)sc_grid_idx(pos.x, P.cell, n), cy = (int)sc_grid_idx(pos.y, P.cell, n),
        cz = (int)sc_grid_idx(pos.z, P.cell, n);
    if (P.periodic) {
        // the z run of a column is one slot range unless it wraps
        for (int ox = R.xl; ox <= R.xh; ox++) {
            for (int oy = R.yl; oy <= R.yh; oy++) {
                uint32_t base = cell_key(P, wrap_cell(cx + ox, n), wrap_cell(cy + oy, n), 0);
                if (cz + R.zl >= 0 && cz + R.zh <= n - 1) {
                    for (uint32_t j = cellStart[base + (uint32_t)(cz + R.zl)],
                                  e = cellStart[(base + (uint32_t)(cz + R.zh)) + 1];
                         j < e; j++)
                        f((int)j);
                } else {
                    for (int oz = R.zl; oz <= R.zh; oz++) {
                        uint32_t key = base + wrap_cell(cz + oz, n);
                        for (uint32_t j = cellStart[key], e = cellStart[key + 1]; j < e; j++) f((int)j);
                    }
                }
            }
        }
        return;
    }
    int x0 = max(cx + R.xl, 0), x1 = min(cx + R.xh, n - 1);
    int y0 = max(cy + R.yl, 0), y1 = min(cy + R.yh, n - 1);
    uint32_t z0 = (uint32_t)max(cz + R.zl, 0), z1 = (uint32_t)min(cz + R.zh, n - 1);
    for (int gx = x0; gx <= x1; gx++) {
        for (int gy = y0; gy <= y1; gy++) {
            uint32_t base = cell_key(P, (uint32_t)gx, (uint32_t)gy, 0);
            uint32_t s = cellStart[base + z0], e = cellStart[(base + z1) + 1];
            for (uint32_t j = s; j < e; j++) f((int)j);
        }
    }
}
template <class F>
__device__ __forceinline__ void scan27(const ScParams &P, const uint32_t *__restrict__ cellStart, sc_f3 pos, F &&f) {
    scan27(P, cellStart, pos, Reach(), f);
}

// Same neighbourhood, one cell at a time (for kernels that interleave two
// arrays cell by cell, metabolites.cuh:174-248).
template <class F>
__device__ __forceinline__ void cells27(const ScParams &P, sc_f3 pos, const Reach &R, F &&f) {
    int n = cell_limit(P);
    int cx = (int)sc_grid_idx(pos.x, P.cell, n), cy = (int)sc_grid_idx(pos.y, P.cell, n),
        cz = (int)sc_grid_idx(pos.z, P.cell, n);
    if (P.periodic) {
        for (int ox = R.xl; ox <= R.xh; ox++)
            for (int oy = R.yl; oy <= R.yh; oy++)
                for (int oz = R.zl; oz <= R.zh; oz++)
                    f(cell_key(P, wrap_cell(cx + ox, n), wrap_cell(cy + oy, n),
                               wrap_cell(cz + oz, n)));
        return;
    }
    for (int gx = max(cx + R.xl, 0); gx <= min(cx + R.xh, n - 1); gx++)
        for (int gy = max(cy + R.yl, 0); gy <= min(cy + R.yh, n - 1); gy++)
            for (int gz = max(cz + R.zl, 0); gz <= min(cz + R.zh, n - 1); gz++)
                f(cell_key(P, (uint32_t)gx, (uint32_t)gy, (uint32_t)gz));
}
template <class F>
__device__ __forceinline__ void cells27(const ScParams &P, sc_f3 pos, F &&f) {
    cells27(P, pos, Reach(), f);
}

__device__ __forceinline__ void set_error(ScCounters *c, int code) { atomicCAS(&c->error, 0, code); }
