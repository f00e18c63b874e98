// sc_grid.cu -- grid binning of the step on sm_103a (grid.cuh:13-139 of the
// reference, whose version is updateIndices -> CUB SortPairs of the whole
// 256/304-byte struct over all 32 key bits -> memset + updateGridRanges).
//
// Here:
//   1. k_sort_keys: cell key of every slot (inactive -> all-ones in the used
//      bits) and the digit histograms of every pass, one read of pos + info;
//   2. k_onesweep: one LSD pass per 8-bit digit over only the 3*bits+1 key bits
//      (Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix
//      Sort for GPUs", 2022): each CTA ranks a 4096-key tile stably in shared
//      memory, publishes its digit counts, resolves its global offsets by a
//      decoupled look-back over predecessor tiles, and scatters (key, slot);
//      sorting the used bits only is the same total order as CUB's 32-bit
//      stable sort, so the permutation is identical;
//   3. k_cell_start: exclusive cell-start table (cells + 1 entries), which is
//      the reference's gridRanges [start, end) for every non-empty cell;
//   4. k_gather_*: every SoA field moved by the permutation.
#include "sc_launch.h"

#define SORT_IPT 16
#define SORT_TILE (SC_THREADS * SORT_IPT)
#define LB_AGG 0x40000000u
#define LB_INC 0x80000000u
#define LB_FLAGS 0xC0000000u
#define LB_VALUE 0x3FFFFFFFu
#define LB_SPIN_LIMIT (1 << 22)

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// In a batched sim the key is the item's replica's key base plus its cell
// in that replica's grid: replicas sort into consecutive key ranges.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_sort_keys(const float4 *__restrict__ pos, const int4 *__restrict__ info,
                                                          int n, ScParams P, uint32_t inactiveKey, int passes,
                                                          uint32_t *__restrict__ keys, uint32_t *__restrict__ hist) {
    __shared__ uint32_t sh[4 * 256];
    for (int t = threadIdx.x; t < passes * 256; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        uint32_t k = inactiveKey;
        const int4 in = info[i];
        if (in.z & SC_ACTIVE) {
            rep_apply<BATCH>(P, in.w);
            sc_f3 p = ld3(pos, i);
            int lim = cell_limit(P);
            k = cell_key(P, sc_grid_idx(p.x, P.cell, lim), sc_grid_idx(p.y, P.cell, lim), sc_grid_idx(p.z, P.cell, lim));
        }
        keys[i] = k;
        for (int d = 0; d < passes; d++) atomicAdd(&sh[d * 256 + ((k >> (8 * d)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < passes * 256; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

// Exclusive scan of 256 values held one per thread (block of 256).
__device__ __forceinline__ uint32_t block_exclusive_scan256(uint32_t v, uint32_t *warp_sums) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; w++) pre += warp_sums[w];
    return pre + x - v;
}

__global__ void __launch_bounds__(SC_THREADS) k_onesweep(const uint32_t *__restrict__ keysIn,
                                                         const uint32_t *__restrict__ valsIn,
                                                         uint32_t *__restrict__ keysOut, uint32_t *__restrict__ valsOut,
                                                         int n, int shift, const uint32_t *__restrict__ hist,
                                                         uint32_t *__restrict__ lookback, int *tileCounter,
                                                         ScCounters *ctr) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_bin[256];
    __shared__ uint32_t s_cnt[8][256];
    __shared__ uint32_t s_off[8][256];
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_wsum[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (uint32_t)atomicAdd(tileCounter, 1);
    s_bin[tid] = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) s_cnt[w][tid] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const long long base = (long long)tile * SORT_TILE;
    const uint32_t ltmask = (1u << lane) - 1u;

    uint32_t key[SORT_IPT], val[SORT_IPT], rank[SORT_IPT];
#pragma unroll
    for (int r = 0; r < SORT_IPT; r++) {
        long long idx = base + r * SC_THREADS + tid;
        if (idx < n) {
            key[r] = keysIn[idx];
            val[r] = valsIn ? valsIn[idx] : (uint32_t)idx;
        } else {
            key[r] = 0;
            val[r] = 0;
        }
    }
    // Stable ranking: tile order is (round, thread); within a round the warp
    // match gives the rank among equal digits, and the per-digit running sum
    // over warps and rounds gives the offset.
#pragma unroll
    for (int r = 0; r < SORT_IPT; r++) {
        bool valid = base + r * SC_THREADS + tid < n;
        uint32_t d = valid ? ((key[r] >> shift) & 0xffu) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t wrank = __popc(peers & ltmask);
        if (valid && wrank == 0) s_cnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_bin[tid];
#pragma unroll
            for (int w = 0; w < 8; w++) {
                uint32_t c = s_cnt[w][tid];
                s_cnt[w][tid] = 0;
                s_off[w][tid] = run;
                run += c;
            }
            s_bin[tid] = run;
        }
        __syncthreads();
        rank[r] = valid ? s_off[warp][d] + wrank : 0u;
    }
    // Decoupled look-back: thread tid owns digit tid.
    const uint32_t cnt = s_bin[tid];
    uint32_t excl = 0;
    if (tile == 0) {
        st_relaxed(&lookback[tid], LB_INC | cnt);
    } else {
        st_relaxed(&lookback[(size_t)tile * 256 + tid], LB_AGG | cnt);
        long long pred = (long long)tile - 1;
        while (pred >= 0) {
            uint32_t v = 0;
            int spins = 0;
            while (true) {
                v = ld_relaxed(&lookback[(size_t)pred * 256 + tid]);
                if (v & LB_FLAGS) break;
                if (++spins > LB_SPIN_LIMIT) {
                    set_error(ctr, SC_DERR_LOOKBACK_TIMEOUT);
                    v = LB_INC;
                    break;
                }
                __nanosleep(32);
            }
            excl += v & LB_VALUE;
            if (v & LB_INC) break;
            pred--;
        }
        st_relaxed(&lookback[(size_t)tile * 256 + tid], LB_INC | (excl + cnt));
    }
    uint32_t gofs = block_exclusive_scan256(hist[tid], s_wsum);
    s_base[tid] = gofs + excl;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < SORT_IPT; r++) {
        long long idx = base + r * SC_THREADS + tid;
        if (idx < n) {
            uint32_t d = (key[r] >> shift) & 0xffu;
            uint32_t dst = s_base[d] + rank[r];
            keysOut[dst] = key[r];
            valsOut[dst] = val[r];
        }
    }
}

// cellStart[c] = first sorted slot whose key >= c, for c in [0, cells];
// inactive keys (>= cells) count as cells.  One binary search per cell.
__global__ void k_cell_start(const uint32_t *__restrict__ keys, int n, uint32_t cells, uint32_t *__restrict__ cellStart) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > (long long)cells) return;
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        uint32_t k = keys[mid];
        if ((long long)k < c) lo = mid + 1;
        else hi = mid;
    }
    cellStart[c] = (uint32_t)lo;
}

// The gathers load every field of the source slot before storing any: the
// destination arrays are other buffers, but the compiler cannot know that,
// and interleaved loads and stores would keep one load in flight per thread.
__global__ void __launch_bounds__(SC_THREADS) k_gather_particles(const uint32_t *__restrict__ perm, int n, PFields src,
                                                                 PFields dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = (int)perm[i];
    const float4 pos = src.pos[s], vel = src.vel[s], rot = src.rot[s], angvel = src.angvel[s];
    const float4 posnoise = src.posnoise[s], angnoise = src.angnoise[s], dbg = src.dbg[s];
    const int4 info = src.info[s];
    const int state = src.state[s], lscs = src.lscs[s], spoly = src.spoly[s], nb = src.nb[s];
    dst.pos[i] = pos;
    dst.vel[i] = vel;
    dst.rot[i] = rot;
    dst.angvel[i] = angvel;
    dst.posnoise[i] = posnoise;
    dst.angnoise[i] = angnoise;
    dst.dbg[i] = dbg;
    dst.info[i] = info;
    dst.state[i] = state;
    dst.lscs[i] = lscs;
    dst.spoly[i] = spoly;
    dst.nb[i] = nb;
    int nw = min(max(nb, 0), SC_MAX_ACTIVE_INTERACTIONS) * 3;
    const int *b = src.bonds + (size_t)s * 24;
    int *o = dst.bonds + (size_t)i * 24;
    for (int k = 0; k < nw; k++) o[k] = b[k];
}

// One step of the metabolic gather: optionally the two double-buffered
// fields (vel, met) into their other buffers, one single-buffer 16-byte field
// and one single-buffer int field into their spares (null: not gathered).
__global__ void __launch_bounds__(SC_THREADS) k_gather_mfield(const uint32_t *__restrict__ perm, int n, int sp4,
                                                              const float4 *__restrict__ vel, float4 *__restrict__ vel2,
                                                              const float4 *__restrict__ met, float4 *__restrict__ met2,
                                                              const float4 *__restrict__ a, float4 *__restrict__ a2,
                                                              const int *__restrict__ c, int *__restrict__ c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = (int)perm[i];
    float4 v = make_float4(0, 0, 0, 0), x = make_float4(0, 0, 0, 0), mt[3];
    int y = 0;
    if (vel) v = vel[s];
    if (a) x = a[s];
    if (c) y = c[s];
#pragma unroll
    for (int k = 0; k < 3; k++)
        if (met && k < sp4) mt[k] = met[(size_t)s * sp4 + k];
    if (vel) vel2[i] = v;
    if (a) a2[i] = x;
    if (c) c2[i] = y;
#pragma unroll
    for (int k = 0; k < 3; k++)
        if (met && k < sp4) met2[(size_t)i * sp4 + k] = mt[k];
}

// ---- host-side launchers -----------------------------------------------------

int sc_sort_passes(int bits) { return (3 * bits + 1 + 7) / 8; }
int sc_sort_passes_for(const ScParams &P) { return ((P.keyBits > 0 ? P.keyBits : 3 * P.bits + 1) + 7) / 8; }

size_t sc_sort_lookback_words(int cap) { return (size_t)((cap + SORT_TILE - 1) / SORT_TILE) * 256; }

// Sorts the keys of one item set; returns the buffer index (0/1) holding the
// sorted keys and the permutation.  hist: 4*256 words, lookback: per pass.
int sc_launch_sort(cudaStream_t st, const float4 *pos, const int4 *info, int n, const ScParams &P,
                   uint32_t *keys[2], uint32_t *vals[2], uint32_t *hist, uint32_t *lookback, ScCounters *ctr,
                   long long *launches) {
    int passes = sc_sort_passes_for(P);
    int keyBits = P.keyBits > 0 ? P.keyBits : 3 * P.bits + 1;
    uint32_t inactiveKey = keyBits >= 32 ? 0xffffffffu : ((1u << keyBits) - 1u);
    int tiles = (n + SORT_TILE - 1) / SORT_TILE;
    size_t lbWords = (size_t)tiles * 256;
    cudaMemsetAsync(hist, 0, 4 * 256 * sizeof(uint32_t), st);
    cudaMemsetAsync(lookback, 0, (size_t)passes * lbWords * sizeof(uint32_t), st);
    cudaMemsetAsync(ctr->tileCounter, 0, sizeof(ctr->tileCounter), st);
    int blocks = (n + SC_THREADS - 1) / SC_THREADS;
    if (n > 0) {
        (P.nRep > 1 ? k_sort_keys<true> : k_sort_keys<false>)<<<blocks, SC_THREADS, 0, st>>>(
            pos, info, n, P, inactiveKey, passes, keys[0], hist);
        (*launches)++;
    }
    int cur = 0;
    for (int d = 0; d < passes && n > 0; d++) {
        k_onesweep<<<tiles, SC_THREADS, 0, st>>>(keys[cur], d == 0 ? nullptr : vals[cur], keys[1 - cur],
                                                  vals[1 - cur], n, 8 * d, hist + 256 * d,
                                                  lookback + (size_t)d * lbWords, &ctr->tileCounter[d], ctr);
        (*launches)++;
        cur = 1 - cur;
    }
    return cur;
}

void sc_launch_cell_start(cudaStream_t st, const uint32_t *keys, int n, uint32_t cells, uint32_t *cellStart,
                          long long *launches) {
    long long total = (long long)cells + 1;
    int blocks = (int)((total + SC_THREADS - 1) / SC_THREADS);
    k_cell_start<<<blocks, SC_THREADS, 0, st>>>(keys, n, cells, cellStart);
    (*launches)++;
}

void sc_launch_gather_particles(cudaStream_t st, const uint32_t *perm, int n, const PFields &src, const PFields &dst,
                                long long *launches) {
    if (n <= 0) return;
    k_gather_particles<<<(n + SC_THREADS - 1) / SC_THREADS, SC_THREADS, 0, st>>>(perm, n, src, dst);
    (*launches)++;
}

// The metabolic gather through the spares (ScBuffers::mChain4 / mChain1):
// from parity 0 field k moves from chain entry k + 1 to entry k, fields in
// ascending order; from parity 1 from entry k to k + 1, in descending order
// (each launch writes the buffer the previous one read).  vel and met go to
// their other buffers in the first launch.  Flips the parity and the two
// double-buffered fields.
void sc_launch_gather_metabolic(cudaStream_t st, const uint32_t *perm, int n, int sp4, ScBuffers &B,
                                long long *launches) {
    if (n > 0) {
        const MFields src = B.M(), dst = B.Mnext();
        const int par = B.mParity;
        for (int t = 0; t < ScBuffers::kM4; t++) {
            const int k = par ? ScBuffers::kM4 - 1 - t : t;
            const float4 *a = par ? B.mChain4[k] : B.mChain4[k + 1];
            float4 *a2 = par ? B.mChain4[k + 1] : B.mChain4[k];
            const int *c = nullptr;
            int *c2 = nullptr;
            if (t < ScBuffers::kM1) {
                const int q = par ? ScBuffers::kM1 - 1 - t : t;
                c = par ? B.mChain1[q] : B.mChain1[q + 1];
                c2 = par ? B.mChain1[q + 1] : B.mChain1[q];
            }
            k_gather_mfield<<<(n + SC_THREADS - 1) / SC_THREADS, SC_THREADS, 0, st>>>(
                perm, n, sp4, t == 0 ? src.vel : nullptr, dst.vel, t == 0 ? src.met : nullptr, dst.met, a, a2, c, c2);
            (*launches)++;
        }
    }
    B.setMParity(1 - B.mParity);
    B.cm[FM_VEL] ^= 1;
    B.cm[FM_MET] ^= 1;
}
