// sc_observe.cu -- ensemble observables reduced in double precision: mean
// squared displacement from a marked origin, mean |v|^2, active and bond
// counts, metabolite totals, and the pair-distance histogram (the radial
// distribution before normalisation).  No counterpart in the reference; the
// long sums are the ones that need FP64.
//
// Every reduction runs in a fixed order: a fixed grid strides over the
// slots, each block reduces its threads' partial sums by a fixed tree into
// one row of a partials table, and one block sums the rows in block order,
// so repeated calls on the same state give the same bytes.
#include "sc_launch.h"

namespace {

constexpr int OBS_BLOCKS = 512;

// Row layout of the partials table.
enum { O_MSD, O_MSD_N, O_V2, O_ACTIVE, O_BONDS, O_MET, O_COLS = O_MET + SC_AOS_NUM_METABOLITES };

__device__ __forceinline__ double min_image(double d, double box, bool periodic) {
    return periodic ? d - box * rint(d / box) : d;
}

// Block reduction of v (one value per thread) in a fixed tree; thread 0 gets the sum.
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < SC_THREADS / 32; w++) s += sh[w];
    __syncthreads();
    return s;
}

// One pass over a set's slots: partial sums of one block into row blockIdx.x.
__global__ void __launch_bounds__(SC_THREADS) k_observe(const int *__restrict__ nActivePtr,
                                                        const float4 *__restrict__ pos,
                                                        const float4 *__restrict__ vel,
                                                        const int4 *__restrict__ info,
                                                        const int *__restrict__ nb, const float *__restrict__ met,
                                                        int sp, int S, const float4 *__restrict__ mark, int markCap,
                                                        double box, int periodic, double *__restrict__ partials) {
    __shared__ double sh[SC_THREADS / 32];
    double acc[O_COLS];
#pragma unroll
    for (int c = 0; c < O_COLS; c++) acc[c] = 0.0;
    const int n = *nActivePtr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 in = info[i];
        if (!(in.z & SC_ACTIVE)) continue;
        acc[O_ACTIVE] += 1.0;
        const float4 p = pos[i], v = vel[i];
        acc[O_V2] += ((double)v.x * v.x + (double)v.y * v.y) + (double)v.z * v.z;
        if (mark && in.x >= 0 && in.x < markCap) {
            const float4 m = mark[in.x];
            if (m.w != 0.0f) {
                const double dx = min_image((double)p.x - (double)m.x, box, periodic != 0);
                const double dy = min_image((double)p.y - (double)m.y, box, periodic != 0);
                const double dz = min_image((double)p.z - (double)m.z, box, periodic != 0);
                acc[O_MSD] += (dx * dx + dy * dy) + dz * dz;
                acc[O_MSD_N] += 1.0;
            }
        }
        if (nb) acc[O_BONDS] += (double)min(max(nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
        if (met)
            for (int s = 0; s < S; s++) acc[O_MET + s] += (double)met[(size_t)i * sp + s];
    }
    for (int c = 0; c < O_COLS; c++) {
        const double t = block_sum(acc[c], sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * O_COLS + c] = t;
    }
}

// Column sums of the partials table, rows in order.
__global__ void k_observe_total(const double *__restrict__ partials, int rows, double *__restrict__ out) {
    const int c = threadIdx.x;
    if (c >= O_COLS) return;
    double s = 0.0;
    for (int r = 0; r < rows; r++) s += partials[(size_t)r * O_COLS + c];
    out[c] = s;
}

__global__ void __launch_bounds__(SC_THREADS) k_mark(const int *__restrict__ nActivePtr, const float4 *__restrict__ pos,
                                                     const int4 *__restrict__ info, float4 *__restrict__ mark,
                                                     int markCap) {
    const int n = *nActivePtr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 in = info[i];
        if ((in.z & SC_ACTIVE) && in.x >= 0 && in.x < markCap) {
            const float4 p = pos[i];
            mark[in.x] = make_float4(p.x, p.y, p.z, 1.0f);
        }
    }
}

// Ordered pairs (i, j), i != j, of the requested types closer than rMax,
// binned by distance; the neighbourhood is the 27 cells of i's cell (rMax is
// at most the cell size, so no pair is missed).  Counts are gathered per
// block in shared memory and added to the global histogram once.
__global__ void __launch_bounds__(SC_THREADS) k_pair_histogram(ScParams P, const uint32_t *__restrict__ cellStart,
                                                               const int *__restrict__ nActivePtr,
                                                               const float4 *__restrict__ pos,
                                                               const int4 *__restrict__ info, int typeA, int typeB,
                                                               double rMax, int nBins,
                                                               unsigned long long *__restrict__ counts) {
    extern __shared__ unsigned long long hist[];
    for (int b = threadIdx.x; b < nBins; b += blockDim.x) hist[b] = 0ull;
    __syncthreads();
    const int n = *nActivePtr;
    const double box = P.simSize, r2max = rMax * rMax;
    const bool periodic = P.periodic != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 in = info[i];
        if (!(in.z & SC_ACTIVE) || (typeA >= 0 && in.y != typeA)) continue;
        const float4 p4 = pos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        scan27(P, cellStart, pp, [&](int j) {
            if (j == i) return;
            const int4 tin = info[j];
            if (!(tin.z & SC_ACTIVE) || (typeB >= 0 && tin.y != typeB)) return;
            const float4 t4 = pos[j];
            const double dx = min_image((double)t4.x - (double)p4.x, box, periodic);
            const double dy = min_image((double)t4.y - (double)p4.y, box, periodic);
            const double dz = min_image((double)t4.z - (double)p4.z, box, periodic);
            const double r2 = (dx * dx + dy * dy) + dz * dz;
            if (r2 < r2max) {
                const int b = (int)(sqrt(r2) * (double)nBins / rMax);
                if (b < nBins) atomicAdd(&hist[b], 1ull);
            }
        });
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nBins; b += blockDim.x)
        if (hist[b]) atomicAdd(&counts[b], hist[b]);
}

}  // namespace

void sc_launch_mark(cudaStream_t st, const int *nActive, const float4 *pos, const int4 *info, float4 *mark,
                    int markCap) {
    k_mark<<<OBS_BLOCKS, SC_THREADS, 0, st>>>(nActive, pos, info, mark, markCap);
}

int sc_observe_cols() { return O_COLS; }
int sc_observe_rows() { return OBS_BLOCKS; }

void sc_launch_observe(cudaStream_t st, const int *nActive, const float4 *pos, const float4 *vel, const int4 *info,
                       const int *nb, const float *met, int sp, int S, const float4 *mark, int markCap, double box,
                       int periodic, double *partials, double *out) {
    k_observe<<<OBS_BLOCKS, SC_THREADS, 0, st>>>(nActive, pos, vel, info, nb, met, sp, S, mark, markCap, box,
                                                  periodic, partials);
    k_observe_total<<<1, 32, 0, st>>>(partials, OBS_BLOCKS, out);
}

void sc_launch_pair_histogram(cudaStream_t st, const ScParams &P, const uint32_t *cellStart, const int *nActive,
                              const float4 *pos, const int4 *info, int typeA, int typeB, double rMax, int nBins,
                              unsigned long long *counts, int gridCap) {
    k_pair_histogram<<<gridCap, SC_THREADS, (size_t)nBins * sizeof(unsigned long long), st>>>(
        P, cellStart, nActive, pos, info, typeA, typeB, rMax, nBins, counts);
}
