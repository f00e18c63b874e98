// sc_noalloc.cu -- a cell sort that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: a host framework that
// has reserved the GPU's memory up front for its own pool (a serving process
// that budgets HBM across requests), or a latency-sensitive loop that cannot
// absorb the device-wide synchronisation cudaMalloc / cudaFree imply.  For
// them, sc_sort_cells_static runs the same binning as a sim's sort (cell key,
// onesweep radix passes, cell-start table) on buffers the caller owns, with
// its working memory in one file-scope static device array of fixed size.
//
// Limits and sharing:
//   * at most SC_STATIC_SORT_MAX_ITEMS items per call (larger calls are
//     rejected with SC_E_INVALID before anything is launched);
//   * the array occupies about 4.3 MB on every GPU that loads the library,
//     until the process exits;
//   * every call on a device uses the same array, so calls whose work
//     overlaps on the GPU (other streams, other host threads) race: order
//     them on one stream, or wait for one to finish before the next starts;
//   * the counters that must start at zero (histograms, look-back words, tile
//     counters, error flag) are cleared by each call; the rest is written
//     before it is read;
//   * every call looks up the array's device address on the current device
//     (a symbol lookup, no allocation; an address kept from an earlier call
//     could be stale after a device reset) and waits for its own results
//     before returning, so it is synchronous and cannot be made while the
//     stream is being captured into a CUDA graph.
#include <string.h>

#include "sc_launch.h"

#define SC_STATIC_SORT_MAX_ITEMS (1 << 18)
#define SC_STATIC_SORT_TILE 4096
#define SC_STATIC_SORT_TILES ((SC_STATIC_SORT_MAX_ITEMS + SC_STATIC_SORT_TILE - 1) / SC_STATIC_SORT_TILE)

namespace {

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t kWords = SC_STATIC_SORT_MAX_ITEMS;
constexpr size_t kKeysOff = 0;                                    // uint32 keys[2][MAX]
constexpr size_t kValsOff = kKeysOff + 2 * kWords * 4;            // uint32 vals[2][MAX]
constexpr size_t kHistOff = kValsOff + 2 * kWords * 4;            // uint32 hist[4][256]
constexpr size_t kLookOff = kHistOff + 4 * 256 * 4;               // uint32 lookback[4][tiles][256]
constexpr size_t kCtrOff = kLookOff + (size_t)4 * SC_STATIC_SORT_TILES * 256 * 4;  // ScCounters
constexpr size_t kBytes = ((kCtrOff + sizeof(ScCounters) + 255) / 256) * 256;

static __device__ __align__(256) unsigned char g_sort_scratch[kBytes];

}  // namespace

extern "C" int sc_sort_cells_static(const sc_config *cfg, const void *pos, const void *info, int32_t n,
                                    uint32_t *perm, uint32_t *cell_start, void *stream) {
    if (!cfg || (n > 0 && (!pos || !info || !perm)) || !cell_start) return SC_E_INVALID;
    if (n < 0 || n > SC_STATIC_SORT_MAX_ITEMS)
        return SC_E_INVALID;
    int32_t ngrid = 0, bits = 0;
    if (sc_config_grid(cfg, &ngrid, &bits) != SC_OK) return SC_E_INVALID;
    // The array's address on the current device: host code sees only a host
    // stand-in of g_sort_scratch, which no kernel may be given.
    void *base = nullptr;
    if (cudaGetSymbolAddress(&base, g_sort_scratch) != cudaSuccess || !base) return SC_E_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    uint32_t *keys[2] = {(uint32_t *)(b + kKeysOff), (uint32_t *)(b + kKeysOff) + kWords};
    uint32_t *vals[2] = {(uint32_t *)(b + kValsOff), (uint32_t *)(b + kValsOff) + kWords};
    uint32_t *hist = (uint32_t *)(b + kHistOff);
    uint32_t *lookback = (uint32_t *)(b + kLookOff);
    ScCounters *ctr = (ScCounters *)(b + kCtrOff);

    ScParams P;
    memset(&P, 0, sizeof P);
    P.cell = cfg->grid_cell_size;
    P.ngrid = ngrid;
    P.bits = bits;
    P.cells = (uint32_t)ngrid * (uint32_t)ngrid * (uint32_t)ngrid;
    P.periodic = cfg->periodic != 0;
    P.walls = cfg->walls != 0;
    P.nUsed = (int)ceilf(cfg->grid_cell_size > 0.0f ? cfg->sim_size / cfg->grid_cell_size : 0.0f);
    if (cfg->periodic && cfg->grid_cell_size > 0.0f)
        P.nUsed = sc_periodic_cells(cfg->sim_size, cfg->grid_cell_size, &P.cell);
    long long launches = 0;
    if (cudaMemsetAsync(ctr, 0, sizeof(ScCounters), st) != cudaSuccess) return SC_E_CUDA;
    int cur = sc_launch_sort(st, (const float4 *)pos, (const int4 *)info, n, P, keys, vals, hist, lookback, ctr,
                             &launches);
    sc_launch_cell_start(st, keys[cur], n, P.cells, cell_start, &launches);
    if (n > 0 && cudaMemcpyAsync(perm, vals[cur], (size_t)n * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return SC_E_CUDA;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return SC_E_CUDA;
    int derr = 0;
    e = cudaMemcpyAsync(&derr, &ctr->error, sizeof derr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return SC_E_CUDA;
    if (derr) return SC_E_DEVICE;
    return SC_OK;
}
