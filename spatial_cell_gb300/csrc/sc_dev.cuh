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

// Device-side error codes (sticky, first one wins).
#define SC_DERR_LOOKBACK_TIMEOUT 1
#define SC_DERR_POLY_OVERFLOW 2

struct ScCounters {
    int nActive;      // nActiveParticles (main.cu:244), bound of every particle kernel
    int lastActive;   // lastActiveParticle (main.cu:245)
    int nextId;       // nextParticleId (main.cu:246)
    int nActiveM;     // nActiveMetabolicParticles (main.cu:253)
    int error;        // first device-side error code
    int polyCount;    // scheduled polymerisations collected this step
    int step;         // the step loop counter (main.cu:347)
    int tileCounter[4];
};

struct ScParams {
    float simSize, maxInt, maxDiff, cell;
    int ngrid, bits;
    uint32_t cells;
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
    return (gx << (2 * P.bits)) | (gy << P.bits) | gz;
}

// Visits the reference's 27-cell neighbourhood of pos (grid.cuh:13-25 and the
// loop of e.g. dynamics.cuh:445-451): cells clamped at the box edge, in gx, gy,
// gz order, slots ascending inside a cell.  Keys of the cells (gx, gy, z0..z1)
// are consecutive, so with the exclusive cell-start table (cellStart[c] =
// first sorted slot with key >= c) that run of cells is one slot range, and
// the visiting order is exactly the reference's.
template <class F>
__device__ __forceinline__ void scan27(const ScParams &P, const uint32_t *__restrict__ cellStart, sc_f3 pos, F &&f) {
    int n = P.ngrid;
    int cx = (int)sc_grid_idx(pos.x, P.cell, n), cy = (int)sc_grid_idx(pos.y, P.cell, n),
        cz = (int)sc_grid_idx(pos.z, P.cell, n);
    int x0 = max(cx - 1, 0), x1 = min(cx + 1, n - 1);
    int y0 = max(cy - 1, 0), y1 = min(cy + 1, n - 1);
    uint32_t z0 = (uint32_t)max(cz - 1, 0), z1 = (uint32_t)min(cz + 1, n - 1);
    for (int gx = x0; gx <= x1; gx++) {
        for (int gy = y0; gy <= y1; gy++) {
            uint32_t base = cell_key(P, (uint32_t)gx, (uint32_t)gy, 0);
            uint32_t s = cellStart[base | z0], e = cellStart[(base | z1) + 1];
            for (uint32_t j = s; j < e; j++) f((int)j);
        }
    }
}

// Same neighbourhood, one cell at a time (for kernels that interleave two
// arrays cell by cell, metabolites.cuh:174-248).
template <class F>
__device__ __forceinline__ void cells27(const ScParams &P, sc_f3 pos, F &&f) {
    int n = P.ngrid;
    int cx = (int)sc_grid_idx(pos.x, P.cell, n), cy = (int)sc_grid_idx(pos.y, P.cell, n),
        cz = (int)sc_grid_idx(pos.z, P.cell, n);
    for (int gx = max(cx - 1, 0); gx <= min(cx + 1, n - 1); gx++)
        for (int gy = max(cy - 1, 0); gy <= min(cy + 1, n - 1); gy++)
            for (int gz = max(cz - 1, 0); gz <= min(cz + 1, n - 1); gz++)
                f(cell_key(P, (uint32_t)gx, (uint32_t)gy, (uint32_t)gz));
}

__device__ __forceinline__ void set_error(ScCounters *c, int code) { atomicCAS(&c->error, 0, code); }
