// sc_tile.cuh -- column-segment tiles for the metabolic neighbour sweeps.
//
// A tile block owns the items of SC_TILE_TX x SC_TILE_TY cell columns over
// SC_TILE_SZ cells of z.  Every cell those items' 27-cell neighbourhoods can
// reach -- (TX+2) x (TY+2) columns over SZ+2 cells, plus in a periodic box
// the cell across the z faces -- lies in a few contiguous slot ranges of the
// sorted arrays (one run per column: keys are x<<2b | y<<b | z).  The block
// copies those ranges into shared memory with bulk asynchronous copies
// (cp.async.bulk, completion counted on an mbarrier), so pair lists name
// neighbours by their 16-bit offset in the tile and the sweeps read
// neighbour data from shared memory instead of gathering it from HBM.
//
// The metabolic and particle grids share the cell geometry: a tile has one
// range table per grid.  Tile offsets put the metabolic slots first
// ([0, capM)) and the particle slots after them ([capM, capM + capP)).
#pragma once

#include "sc_dev.cuh"

#define SC_TILE_TX 2
#define SC_TILE_TY 2
#define SC_TILE_SZ 8
#define SC_TILE_NCOL ((SC_TILE_TX + 2) * (SC_TILE_TY + 2))
#define SC_TILE_NRANGE (3 * SC_TILE_NCOL)  // per column: the z run, the cell below z = 0, the cell above the top
#define SC_TILE_NITEMCOL (SC_TILE_TX * SC_TILE_TY)
#define SC_DERR_TILE_TIMEOUT 3

// Cells per axis items can occupy: the cells a periodic box spans, or in a
// walled box those up to the one holding simSize itself.
__host__ __device__ __forceinline__ int tile_axis_cells(const ScParams &P) {
    return P.periodic ? P.nUsed : min(P.nUsed + 1, P.ngrid);
}
__host__ __device__ __forceinline__ int tile_blocks(const ScParams &P) {
    const int n = tile_axis_cells(P);
    return ((n + SC_TILE_TX - 1) / SC_TILE_TX) * ((n + SC_TILE_TY - 1) / SC_TILE_TY) *
           ((n + SC_TILE_SZ - 1) / SC_TILE_SZ);
}

struct TileGeom {
    int n;                 // cells per axis (tile_axis_cells)
    bool periodic;
    int x0, y0, z0, z1;    // item columns x0 + [0, TX), y0 + [0, TY); item cells z in [z0, z1)
    int tz0, tz1;          // the z run of every tile column
    bool wrapLo, wrapHi;   // periodic: the tile also holds cell n-1 (below z0 = 0) / cell 0 (above z1 = n)

    __device__ __forceinline__ void init(const ScParams &P, int blk) {
        n = tile_axis_cells(P);
        periodic = P.periodic != 0;
        const int nbz = (n + SC_TILE_SZ - 1) / SC_TILE_SZ, nby = (n + SC_TILE_TY - 1) / SC_TILE_TY;
        const int bz = blk % nbz, by = (blk / nbz) % nby, bx = blk / (nbz * nby);
        x0 = bx * SC_TILE_TX;
        y0 = by * SC_TILE_TY;
        z0 = bz * SC_TILE_SZ;
        z1 = min(z0 + SC_TILE_SZ, n);
        tz0 = max(z0 - 1, 0);
        tz1 = min(z1 + 1, n);
        wrapLo = periodic && z0 == 0 && tz1 < n;
        wrapHi = periodic && z1 == n && tz0 > 0;
    }
    // Cell column of tile column t (0 .. T+1) along an axis starting at
    // origin; -1 outside a walled box.
    __device__ __forceinline__ int col(int t, int origin) const {
        int c = origin - 1 + t;
        if (c < 0 || c >= n) {
            if (!periodic) return -1;
            c = (c + n) % n;
        }
        return c;
    }
    // Tile column index of cell column (x, y), -1 if the tile has none.
    __device__ __forceinline__ int col_index(int x, int y) const {
        int tx = x - (x0 - 1), ty = y - (y0 - 1);
        if (periodic) {  // x, y in [0, n), x0 - 1 in [-1, n - 1): one wrap at most
            tx += tx < 0 ? n : (tx >= n ? -n : 0);
            ty += ty < 0 ? n : (ty >= n ? -n : 0);
        }
        if (tx < 0 || tx >= SC_TILE_TX + 2 || ty < 0 || ty >= SC_TILE_TY + 2) return -1;
        return tx * (SC_TILE_TY + 2) + ty;
    }
    // Range of the tile holding cell (x, y, z), -1 if none.
    __device__ __forceinline__ int range_of(int x, int y, int z) const {
        const int c = col_index(x, y);
        if (c < 0) return -1;
        if (z >= tz0 && z < tz1) return 3 * c;
        if (wrapLo && z == n - 1) return 3 * c + 1;
        if (wrapHi && z == 0) return 3 * c + 2;
        return -1;
    }
    // Slot span [b, b + l) of range r in a grid.
    __device__ __forceinline__ void span(const ScParams &P, const uint32_t *__restrict__ cellStart, int r, int &b,
                                         int &l) const {
        b = 0;
        l = 0;
        const int c = r / 3, kind = r % 3;
        const int gx = col(c / (SC_TILE_TY + 2), x0), gy = col(c % (SC_TILE_TY + 2), y0);
        int za = 0, zb = 0;
        if (kind == 0) { za = tz0; zb = tz1; }
        else if (kind == 1 && wrapLo) { za = n - 1; zb = n; }
        else if (kind == 2 && wrapHi) { za = 0; zb = 1; }
        if (gx < 0 || gy < 0 || zb <= za) return;
        const uint32_t k0 = cell_key(P, (uint32_t)gx, (uint32_t)gy, 0);
        b = (int)cellStart[k0 + (uint32_t)za];
        l = (int)cellStart[k0 + (uint32_t)zb] - b;
    }
};

// The range table of one grid: slot base, slot count (clipped to the
// capacity) and tile offset of each range.
struct TileRanges {
    int base[SC_TILE_NRANGE];
    int len[SC_TILE_NRANGE];
    int off[SC_TILE_NRANGE];
    int total;  // slots the tile needs (above the capacity: it overflowed)
};

// Fills the range table of one grid for the block's tile; run by one whole
// warp.  Offsets start at `first`; slots past `cap` are clipped.
__device__ __forceinline__ void tile_ranges(const ScParams &P, const TileGeom &G,
                                            const uint32_t *__restrict__ cellStart, int first, int cap,
                                            TileRanges &R) {
    const int lane = threadIdx.x & 31;
    int total = 0;
    for (int r0 = 0; r0 < SC_TILE_NRANGE; r0 += 32) {
        const int r = r0 + lane;
        int b = 0, l = 0;
        if (r < SC_TILE_NRANGE) G.span(P, cellStart, r, b, l);
        int x = l;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (r < SC_TILE_NRANGE) {
            const int off = total + x - l;
            R.base[r] = b;
            R.off[r] = first + min(off, cap);
            R.len[r] = max(0, min(l, cap - off));
        }
        total += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) R.total = total;
}

// ---- bulk asynchronous copies into shared memory -----------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// Source and destination 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for phase 0 of the barrier for at most about `cycles` SM clocks.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, long long cycles) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, 0))
        if (clock64() - t0 > cycles) return false;
    return true;
}

// Bytes one float4 field of a grid occupies in the tile.
__device__ __forceinline__ uint32_t tile_field_bytes(const TileRanges &R) {
    uint32_t b = 0;
    for (int r = 0; r < SC_TILE_NRANGE; r++) b += (uint32_t)max(R.len[r], 0) * 16u;
    return b;
}
// Bulk-copies one float4 field of a grid, range by range, into the tile array
// `dst` (indexed by tile offset); issued by one thread.
__device__ __forceinline__ void tile_issue(const TileRanges &R, const float4 *src, float4 *dst, uint64_t *bar) {
    for (int r = 0; r < SC_TILE_NRANGE; r++)
        if (R.len[r] > 0) bulk_copy(dst + R.off[r], src + R.base[r], (uint32_t)R.len[r] * 16u, bar);
}
