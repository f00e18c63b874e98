// sc_sim.cu -- the C ABI of include/spatialcell.h: one sim = its device
// buffers, one CUDA stream and the launch sequence of the step loop
// (main.cu:347-661), with no host synchronisation inside a step.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <map>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <cmath>
#include <string>
#include <vector>

#include "sc_gen.h"
#include "sc_launch.h"
#include "sc_tile.cuh"

extern "C" const char *sc_host_last_error(void);

namespace {

thread_local std::string g_err;

// ---- AoS <-> SoA (device side; the host buffers move in one copy) -----------
// Byte offsets of the reference's Particle (types.cuh:173-222).
__device__ __forceinline__ float4 rd4(const uint8_t *r, int off) { return *(const float4 *)(r + off); }
__device__ __forceinline__ float rdf(const uint8_t *r, int off) { return *(const float *)(r + off); }
__device__ __forceinline__ int rdi(const uint8_t *r, int off) { return *(const int *)(r + off); }
__device__ __forceinline__ int rdb(const uint8_t *r, int off) { return (int)*(const int8_t *)(r + off); }

// Sum of list counts over the active items (counts above a list's capacity
// are overflowed items, counted as they are).
__global__ void k_sum_counts(const int *__restrict__ cnt, const int *__restrict__ nActivePtr, long long *out) {
    const int n = *nActivePtr;
    long long acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc += cnt[i] == INT_MAX ? 0 : cnt[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long *)out, (unsigned long long)acc);
}

// Items of a list whose count is above `limit` (overflowed).
__global__ void k_count_over(const int *__restrict__ cnt, const int *__restrict__ nActivePtr, int limit,
                             long long *out) {
    const int n = *nActivePtr;
    long long acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += cnt[i] > limit;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long *)out, (unsigned long long)acc);
}

__global__ void k_gen_particles(uint8_t *aos, int n, float box, sc_gen_mix mix, uint64_t seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sc_gen_particle(reinterpret_cast<sc_particle *>(aos + (size_t)i * sizeof(sc_particle)), i, box, &mix, seed);
}
// Work unit u of a scene group: its first record is at particle first + u * per.
__global__ void k_gen_scene(uint8_t *aos, sc_gen_group G, int per, float box, uint64_t seed) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < G.count)
        sc_gen_unit(reinterpret_cast<sc_particle *>(aos + (size_t)(G.first + (int64_t)u * per) * sizeof(sc_particle)), &G,
                    u, box, seed);
}
__global__ void k_gen_metabolic(uint8_t *aos, int nm, float box, int species, float radius, int8_t hydrophobic,
                                uint64_t seed) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nm)
        sc_gen_metabolic(reinterpret_cast<sc_metabolic_particle *>(aos + (size_t)j * sizeof(sc_metabolic_particle)), j,
                         box, species, radius, hydrophobic, seed);
}

// Slots [0, cap) of F (records i < n from aos, the rest empty).  With `bad`,
// the lowest record index (plus base) whose interaction count is outside
// 0..8 is recorded there by atomicMin.
__global__ void k_unpack_particles(const uint8_t *__restrict__ aos, int n, int cap, PFields F, int *bad = nullptr,
                                   int base = 0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    if (i >= n) {
        F.pos[i] = F.vel[i] = F.rot[i] = F.angvel[i] = F.posnoise[i] = F.angnoise[i] = F.dbg[i] = make_float4(0, 0, 0, 0);
        F.info[i] = make_int4(0, 0, 0, 0);
        F.state[i] = F.lscs[i] = F.spoly[i] = F.nb[i] = 0;
        return;
    }
    const uint8_t *r = aos + (size_t)i * 256;
    F.info[i] = make_int4(rdi(r, 0), rdi(r, 4), rdi(r, 8), rdb(r, 24));
    F.state[i] = rdb(r, 12);
    F.lscs[i] = rdi(r, 16);
    F.pos[i] = make_float4(rdf(r, 28), rdf(r, 32), rdf(r, 36), rdf(r, 20));
    F.rot[i] = rd4(r, 48);
    F.vel[i] = make_float4(rdf(r, 64), rdf(r, 68), rdf(r, 72), 0.0f);
    F.posnoise[i] = make_float4(rdf(r, 76), rdf(r, 80), rdf(r, 84), 0.0f);
    F.angvel[i] = rd4(r, 96);
    F.angnoise[i] = rd4(r, 112);
    int nb = rdi(r, 128);
    if (bad && (nb < 0 || nb > SC_MAX_ACTIVE_INTERACTIONS)) atomicMin(bad, base + i);
    F.nb[i] = nb;
    for (int k = 0; k < 24; k++) F.bonds[(size_t)i * 24 + k] = k < 3 * min(max(nb, 0), 8) ? rdi(r, 132 + 4 * k) : 0;
    F.spoly[i] = rdi(r, 228);
    F.dbg[i] = rd4(r, 240);
}

// Slots [0, cap) of F (records i < n from aos, the rest empty); `base` is the
// load slot of slot 0 (F shifted to a batch replica's first slot).
__global__ void k_unpack_metabolic(const uint8_t *__restrict__ aos, int n, int cap, int SP, MFields F, int *cLscs,
                                   int *cSpoly, int *cNb, int *cBonds, int base = 0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    F.orig[i] = base + i;
    if (i >= n) {
        F.pos[i] = F.vel[i] = F.rot[i] = F.angvel[i] = F.posnoise[i] = F.angnoise[i] = F.dbg[i] = make_float4(0, 0, 0, 0);
        F.info[i] = make_int4(0, 0, 0, 0);
        F.state[i] = 0;
        if (cLscs) {
            cLscs[i] = cSpoly[i] = cNb[i] = 0;
            for (int k = 0; k < 24; k++) cBonds[(size_t)i * 24 + k] = 0;
        }
        for (int q = 0; q < SP / 4; q++) F.met[(size_t)i * (SP / 4) + q] = make_float4(0, 0, 0, 0);
        return;
    }
    const uint8_t *r = aos + (size_t)i * 304;
    F.info[i] = make_int4(rdi(r, 0), rdi(r, 4), rdi(r, 8), rdb(r, 24));
    F.state[i] = rdb(r, 12);
    F.pos[i] = make_float4(rdf(r, 28), rdf(r, 32), rdf(r, 36), rdf(r, 20));
    F.rot[i] = rd4(r, 48);
    F.vel[i] = make_float4(rdf(r, 64), rdf(r, 68), rdf(r, 72), 0.0f);
    F.posnoise[i] = make_float4(rdf(r, 76), rdf(r, 80), rdf(r, 84), 0.0f);
    F.angvel[i] = rd4(r, 96);
    F.angnoise[i] = rd4(r, 112);
    if (cLscs) {
        cLscs[i] = rdi(r, 16);
        int nb = rdi(r, 128);
        cNb[i] = nb;
        for (int k = 0; k < 24; k++) cBonds[(size_t)i * 24 + k] = k < 3 * min(max(nb, 0), 8) ? rdi(r, 132 + 4 * k) : 0;
        cSpoly[i] = rdi(r, 228);
    }
    F.dbg[i] = rd4(r, 240);
    float *met = (float *)(F.met) + (size_t)i * SP;
    for (int k = 0; k < SP; k++) met[k] = k < SC_AOS_NUM_METABOLITES ? rdf(r, 256 + 4 * k) : 0.0f;
}

// Whether staged metabolic records differ from record 0 in the fields no step
// kernel touches (interaction count, last state-change step, scheduled
// polymerisation): any record with interactions or another value sets *mixed.
__global__ void k_mc_scan(const uint8_t *__restrict__ aos, int n, int *mixed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t *r = aos + (size_t)i * 304;
    if (rdi(r, 128) != 0 || rdi(r, 16) != rdi(aos, 16) || rdi(r, 228) != rdi(aos, 228)) *mixed = 1;
}
// The same test against given values (records loaded chunk by chunk).
__global__ void k_mc_scan_ref(const uint8_t *__restrict__ aos, int n, int lscs0, int spoly0, int *mixed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t *r = aos + (size_t)i * 304;
    if (rdi(r, 128) != 0 || rdi(r, 16) != lscs0 || rdi(r, 228) != spoly0) *mixed = 1;
}

__device__ __forceinline__ void wr4(uint8_t *r, int off, float4 v) { *(float4 *)(r + off) = v; }
__device__ __forceinline__ void wrf(uint8_t *r, int off, float v) { *(float *)(r + off) = v; }
__device__ __forceinline__ void wri(uint8_t *r, int off, int v) { *(int *)(r + off) = v; }

__device__ void pack_common(uint8_t *r, int4 in, int state, int lscs, float4 pos, float4 rot, float4 vel, float4 pn,
                            float4 av, float4 an, int nb, const int *bonds, int spoly, float4 dbg) {
    for (int k = 0; k < 256; k += 16) *(int4 *)(r + k) = make_int4(0, 0, 0, 0);
    wri(r, 0, in.x); wri(r, 4, in.y); wri(r, 8, in.z);
    *(int8_t *)(r + 12) = (int8_t)state;
    wri(r, 16, lscs);
    wrf(r, 20, pos.w);
    *(int8_t *)(r + 24) = (int8_t)in.w;
    wrf(r, 28, pos.x); wrf(r, 32, pos.y); wrf(r, 36, pos.z);
    wr4(r, 48, rot);
    wrf(r, 64, vel.x); wrf(r, 68, vel.y); wrf(r, 72, vel.z);
    wrf(r, 76, pn.x); wrf(r, 80, pn.y); wrf(r, 84, pn.z);
    wr4(r, 96, av);
    wr4(r, 112, an);
    wri(r, 128, nb);
    int nw = 3 * min(max(nb, 0), 8);
    for (int k = 0; k < nw; k++) wri(r, 132 + 4 * k, bonds[k]);
    wri(r, 228, spoly);
    wr4(r, 240, dbg);
}

// Slots [base, end) into records aos[0, end - base).
__global__ void k_pack_particles(uint8_t *__restrict__ aos, const int *nActivePtr, int base, int end, PFields F) {
    const int i = base + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    uint8_t *r = aos + (size_t)(i - base) * 256;
    if (i >= *nActivePtr) {
        for (int k = 0; k < 256; k += 16) *(int4 *)(r + k) = make_int4(0, 0, 0, 0);
        return;
    }
    pack_common(r, F.info[i], F.state[i], F.lscs[i], F.pos[i], F.rot[i], F.vel[i], F.posnoise[i], F.angvel[i],
                F.angnoise[i], F.nb[i], F.bonds + (size_t)i * 24, F.spoly[i], F.dbg[i]);
}

__global__ void k_pack_metabolic(uint8_t *__restrict__ aos, const int *nActivePtr, int base, int end, int SP,
                                 MFields F, const int *cLscs, const int *cSpoly, const int *cNb, const int *cBonds,
                                 int lscs0, int spoly0) {
    const int i = base + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    uint8_t *r = aos + (size_t)(i - base) * 304;
    if (i >= *nActivePtr) {
        for (int k = 0; k < 304; k += 16) *(int4 *)(r + k) = make_int4(0, 0, 0, 0);
        return;
    }
    int o = F.orig[i];
    if (cLscs)
        pack_common(r, F.info[i], F.state[i], cLscs[o], F.pos[i], F.rot[i], F.vel[i], F.posnoise[i], F.angvel[i],
                    F.angnoise[i], cNb[o], cBonds + (size_t)o * 24, cSpoly[o], F.dbg[i]);
    else
        pack_common(r, F.info[i], F.state[i], lscs0, F.pos[i], F.rot[i], F.vel[i], F.posnoise[i], F.angvel[i],
                    F.angnoise[i], 0, nullptr, spoly0, F.dbg[i]);
    for (int k = 256; k < 304; k += 16) *(int4 *)(r + k) = make_int4(0, 0, 0, 0);
    const float *met = (const float *)(F.met) + (size_t)i * SP;
    for (int k = 0; k < SC_AOS_NUM_METABOLITES && k < SP; k++) wrf(r, 256 + 4 * k, met[k]);
}

__global__ void k_after_sort(ScCounters *c) { c->lastActive = c->nActive - 1; }

// The replica of every slot of a batch just loaded: the loaded items are the
// replicas' items one replica after another (offsets: nRep + 1 prefix
// sums); slots past them get the replica id nRep, which names no replica.
__global__ void k_set_reps(int4 *__restrict__ info, int cap, const int *__restrict__ offsets, int nRep) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    int lo = 0, hi = nRep;  // the last replica whose offset is <= i
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const int r = i < offsets[nRep] ? lo : nRep;
    int4 in = info[i];
    in.w = (in.w & 0xff) | (r << 8);
    info[i] = in;
}
// Per sorted particle slot: 1 for an active lipid (the metabolic kernels'
// candidate test); slots past the active ones are cleared.
__global__ void k_mark_lipids(const int *__restrict__ nActivePtr, int cap, const int4 *__restrict__ info,
                              uint8_t *__restrict__ lipid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    const int4 in = info[i];
    lipid[i] = (i < *nActivePtr && (in.z & SC_ACTIVE) && in.y == SC_PARTICLE_TYPE_LIPID) ? 1 : 0;
}
__global__ void k_end_step(ScCounters *c) { c->step++; }

}  // namespace

struct sc_sim {
    sc_config cfg;
    ScParams P;
    ScBuffers B;
    cudaStream_t st = nullptr;
    cudaStream_t copySt = nullptr;          // frame copies to the host
    cudaStream_t side[2] = {nullptr, nullptr};  // concurrent kernels of one phase (ScLaunchCtx)
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    bool forkClasses = false;               // run independent kernels of a phase on the side streams
    cudaEvent_t reduced[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    int64_t frames = 0;                     // frames enqueued by sc_reduce_frame_async
    // One step as a CUDA graph, per host-side buffer state at the step's start
    // (which of each field's two buffers is current, sort buffers, list
    // validity, binning): the graph and the state the step leaves behind.
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        std::vector<int> after;
        long long launches = 0;
    };
    std::map<std::vector<int>, StepGraph> graphs;
    bool useGraphs = true;
    int device = 0;
    int gridCap = 0;
    long long launches = 0;
    std::string err;
    std::vector<void *> allocs;
    std::map<void *, size_t> allocBytes;    // bytes of each allocation in allocs
    int64_t notifyKey = -1;                 // queued when each sc_step's work finishes (sc_set_notify)
    std::vector<sc_type_info> types;        // host copy of the type table
    uint8_t *staging = nullptr;
    size_t stagingBytes = 0;
    bool loaded = false;
    // observables: MSD origins by id, the partials table and the results
    float4 *markP = nullptr, *markM = nullptr;
    int markCapP = 0, markCapM = 0;
    double *obs = nullptr;  // partials table, then 2 result rows
    // batched sims (sc_create_batch): the replicas and their geometry
    std::vector<sc_replica> reps;
    std::vector<ScRep> repGeom;
};

namespace {

int set_err(sc_sim *s, int code, const std::string &m) {
    if (s) s->err = m;
    g_err = m;
    return code;
}

#define SC_CK(s, call)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            cudaGetLastError(); /* reported here: not again by the next launch check */                   \
            return set_err((s), e_ == cudaErrorMemoryAllocation ? SC_E_OOM : SC_E_CUDA,                   \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                           \
        }                                                                                                 \
    } while (0)

// Initial metabolic pair pool entries per item (the pool grows to demand).
const int kPoolStart = 12;

// Device memory comes from the device's stream-ordered pool on the sim's
// stream: creating or destroying a sim does not synchronise the device, so
// sims can come and go while others run (the request loop relies on it).
// Completion notices (sc_set_notify / sc_wait_notices): a host function
// enqueued on a sim's stream after its steps queues the sim's key when the
// device reaches it; waiters block on a condition variable instead of
// polling the streams.  The host function calls no CUDA function.
std::mutex g_noticeMu;
std::condition_variable g_noticeCv;
std::deque<int64_t> g_notices;

void CUDART_CB notice_cb(void *arg) {
    {
        std::lock_guard<std::mutex> lk(g_noticeMu);
        g_notices.push_back((int64_t)(intptr_t)arg);
    }
    g_noticeCv.notify_all();
}

// A device allocation the sim no longer owns (freed by the caller).
void forget_alloc(sc_sim *s, void *p) {
    s->allocs.erase(std::find(s->allocs.begin(), s->allocs.end(), p));
    s->allocBytes.erase(p);
}

template <class T>
int dalloc(sc_sim *s, T **p, size_t count) {
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMallocAsync((void **)p, bytes, s->st);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();  // reported here: not again by the next launch check
        return set_err(s, e == cudaErrorMemoryAllocation ? SC_E_OOM : SC_E_CUDA,
                       "cudaMallocAsync of " + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    }
    s->allocs.push_back((void *)*p);
    s->allocBytes[(void *)*p] = bytes;
    return SC_OK;
}

#define SC_ALLOC(s, p, n)                   \
    do {                                    \
        int rc_ = dalloc((s), &(p), (n));   \
        if (rc_) return rc_;                \
    } while (0)

inline int nb_of(long long n) { return (int)((n + SC_THREADS - 1) / SC_THREADS); }

ScLaunchCtx ctx(sc_sim *s) {
    ScLaunchCtx c;
    c.st = s->st;
    c.P = s->P;
    c.B = &s->B;
    c.launches = &s->launches;
    c.gridCap = s->gridCap;
    c.side[0] = s->forkClasses ? s->side[0] : nullptr;
    c.side[1] = s->forkClasses ? s->side[1] : nullptr;
    c.fork = s->fork;
    c.join[0] = s->join[0];
    c.join[1] = s->join[1];
    return c;
}

// Entry of a call on a sim: its device current, and the runtime's last-error
// slot cleared.  That slot is per thread and shared with every other CUDA
// user in the process; an error left there by someone else's failed call (an
// allocation refused for lack of room) is not one of this sim's launches, and
// every call of this library checks its own results as it makes them.
void enter(const sc_sim *s) {
    cudaSetDevice(s->device);
    cudaGetLastError();
}

int check_launch(sc_sim *s) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(s, SC_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return SC_OK;
}

void sort_particles(sc_sim *s) {
    ScBuffers &B = s->B;
    const int N = s->P.N;
    PFields F = B.P();
    int cur = sc_launch_sort(s->st, F.pos, F.info, N, s->P, B.keysP, B.valsP, B.hist, B.lookback, B.ctr, &s->launches);
    B.sortCurP = cur;
    sc_launch_cell_start(s->st, B.keysP[cur], N, s->P.cells, B.cellStartP, &s->launches);
    sc_launch_gather_particles(s->st, B.valsP[cur], N, B.P(), B.Pnext(), &s->launches);
    B.flipAllP();
    k_after_sort<<<1, 1, 0, s->st>>>(B.ctr);
    k_mark_lipids<<<nb_of(N), SC_THREADS, 0, s->st>>>(&B.ctr->nActive, N, B.P().info, B.lipidP);
    s->launches += 2;
}

void sort_metabolic(sc_sim *s) {
    ScBuffers &B = s->B;
    const int Nm = s->P.Nm;
    MFields F = B.M();
    int cur = sc_launch_sort(s->st, F.pos, F.info, Nm, s->P, B.keysM, B.valsM, B.hist, B.lookback, B.ctr, &s->launches);
    B.sortCurM = cur;
    sc_launch_cell_start(s->st, B.keysM[cur], Nm, s->P.cells, B.cellStartM, &s->launches);
    sc_launch_gather_metabolic(s->st, B.valsM[cur], Nm, s->P.SP / 4, B, &s->launches);
}

// Which pair lists a phase invalidates (it changes positions, flags, types,
// radii or interactions their tests read, or re-sorts slots they index).
void invalidate_after(ScBuffers &B, int phase) {
    switch (phase) {
        case SC_PHASE_SORT_PARTICLES: B.validPP = B.validM = B.validLM = false; break;
        case SC_PHASE_SORT_METABOLIC: B.validM = B.validLM = B.validD = false; break;
        case SC_PHASE_APPLY_VELOCITIES: B.invalidateLists(); break;
        case SC_PHASE_COMPLEXIFY:
        case SC_PHASE_TRANSITION:
        case SC_PHASE_POLYMERIZE: B.validPP = B.validLM = false; break;
        case SC_PHASE_REMOVE_INTERFERING: B.validM = B.validLM = B.validD = false; break;
        default: break;
    }
}

// Which sets still sit in the cells they were sorted into: a sort bins its
// set, moving positions unbins both (particles a polymerisation creates are in
// no cell, so they are never found as neighbours).
void binned_after(ScParams &P, int phase) {
    if (phase == SC_PHASE_SORT_PARTICLES) P.binned |= SC_BINNED_P;
    if (phase == SC_PHASE_SORT_METABOLIC) P.binned |= SC_BINNED_M;
    if (phase == SC_PHASE_APPLY_VELOCITIES) P.binned = 0;
    if (phase == SC_PHASE_SORT_METABOLIC) P.mAllActive = 1;  // inactive items sort past the cells
    if (phase == SC_PHASE_REMOVE_INTERFERING) P.mAllActive = 0;
    if (phase == SC_PHASE_SORT_PARTICLES) P.lipidValid = 1;  // marked by sort_particles
}

// The host-side state a step reads and changes.
std::vector<int> host_state(const sc_sim *s) {
    const ScBuffers &B = s->B;
    std::vector<int> v(B.cp, B.cp + FP_COUNT);
    v.insert(v.end(), B.cm, B.cm + FM_COUNT);
    v.insert(v.end(), {B.sortCurP, B.sortCurM, (int)B.validPP, (int)B.validM, (int)B.validLM, (int)B.validD,
                       s->P.binned, s->P.mAllActive, s->P.lipidValid, B.mParity});
    return v;
}
void set_host_state(sc_sim *s, const std::vector<int> &v) {
    ScBuffers &B = s->B;
    size_t k = 0;
    for (int f = 0; f < FP_COUNT; f++) B.cp[f] = v[k++];
    for (int f = 0; f < FM_COUNT; f++) B.cm[f] = v[k++];
    B.sortCurP = v[k++];
    B.sortCurM = v[k++];
    B.validPP = v[k++] != 0;
    B.validM = v[k++] != 0;
    B.validLM = v[k++] != 0;
    B.validD = v[k++] != 0;
    s->P.binned = v[k++];
    s->P.mAllActive = v[k++];
    s->P.lipidValid = v[k++];
    B.setMParity(v[k++]);
}

int run_phase(sc_sim *s, int phase, int arg) {
    ScLaunchCtx c = ctx(s);
    invalidate_after(s->B, phase);
    binned_after(s->P, phase);
    switch (phase) {
        case SC_PHASE_SORT_PARTICLES: sort_particles(s); break;
        case SC_PHASE_SORT_METABOLIC: sort_metabolic(s); break;
        case SC_PHASE_MOVE_BROWNIAN: sc_phase_move_brownian(c, false); break;
        case SC_PHASE_MOVE_BROWNIAN_METAB: sc_phase_move_brownian(c, true); break;
        case SC_PHASE_COORDINATE_NOISE:
            sc_phase_coordinate_noise(c, (float)arg / s->cfg.noise_coordination_steps);
            break;
        case SC_PHASE_APPLY_NOISE: sc_phase_apply_noise(c); break;
        case SC_PHASE_RELAX: sc_phase_relax(c); break;
        case SC_PHASE_RELAX_METAB: sc_phase_relax_metab(c); break;
        case SC_PHASE_RELAX_PARTNERS: sc_phase_relax_partners(c); break;
        case SC_PHASE_APPLY_VELOCITIES: sc_phase_apply_velocities(c); break;
        case SC_PHASE_COMPLEXIFY: sc_phase_complexify(c, arg == -1); break;
        case SC_PHASE_TRANSITION: sc_phase_transition(c); break;
        case SC_PHASE_POLYMERIZE: sc_phase_polymerize(c); break;
        case SC_PHASE_PROPAGATE_STATE: sc_phase_propagate_state(c); break;
        case SC_PHASE_DIFFUSE: sc_phase_diffuse(c); break;
        case SC_PHASE_REMOVE_INTERFERING: sc_phase_remove_interfering(c); break;
        case SC_PHASE_END_STEP:
            k_end_step<<<1, 1, 0, s->st>>>(s->B.ctr);
            s->launches++;
            break;
        default: return set_err(s, SC_E_INVALID, "unknown phase " + std::to_string(phase));
    }
    return check_launch(s);
}

// One iteration of the step loop (main.cu:347-661), launched phase by phase.
int step_direct(sc_sim *s) {
    const sc_config &c = s->cfg;
    run_phase(s, SC_PHASE_SORT_PARTICLES, 0);
    run_phase(s, SC_PHASE_SORT_METABOLIC, 0);
    run_phase(s, SC_PHASE_MOVE_BROWNIAN, 0);
    run_phase(s, SC_PHASE_MOVE_BROWNIAN_METAB, 0);
    for (int j = 0; j < c.noise_coordination_steps; j++) run_phase(s, SC_PHASE_COORDINATE_NOISE, j);
    run_phase(s, SC_PHASE_APPLY_NOISE, 0);
    for (int j = 0; j < c.relaxation_steps; j++) {
        run_phase(s, SC_PHASE_RELAX, j);
        if (j % 2 == 0) {
            run_phase(s, SC_PHASE_RELAX_METAB, j);
            run_phase(s, SC_PHASE_RELAX_PARTNERS, j);
        }
    }
    run_phase(s, SC_PHASE_APPLY_VELOCITIES, 0);
    run_phase(s, SC_PHASE_COMPLEXIFY, 0);
    run_phase(s, SC_PHASE_TRANSITION, 0);
    run_phase(s, SC_PHASE_POLYMERIZE, 0);
    if (c.propagate_state) run_phase(s, SC_PHASE_PROPAGATE_STATE, 0);
    for (int j = 0; j < c.metabolite_diffusion_steps; j++) run_phase(s, SC_PHASE_DIFFUSE, j);
    return run_phase(s, SC_PHASE_END_STEP, 0);
}

// The same step as one graph launch: the first step from a given host-side
// state is captured and instantiated, later ones relaunch it.  A capture that
// fails turns graphs off for the sim and runs the step directly.
int step_graph(sc_sim *s) {
    const std::vector<int> before = host_state(s);
    auto it = s->graphs.find(before);
    if (it == s->graphs.end()) {
        const long long l0 = s->launches;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? step_direct(s) : SC_E_CUDA;
        cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(s->st, &g) : e;
        if (rc == SC_OK && e2 == cudaSuccess) e2 = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (rc != SC_OK || e2 != cudaSuccess) {
            cudaGetLastError();
            s->useGraphs = false;
            s->launches = l0;
            set_host_state(s, before);
            return step_direct(s);
        }
        sc_sim::StepGraph sg;
        sg.exec = exec;
        sg.after = host_state(s);
        sg.launches = s->launches - l0;
        s->launches = l0;
        it = s->graphs.emplace(before, std::move(sg)).first;
    }
    SC_CK(s, cudaGraphLaunch(it->second.exec, s->st));
    set_host_state(s, it->second.after);
    s->launches += it->second.launches;
    return SC_OK;
}

// Once per device: the default memory pool keeps what sims free for the next
// ones (no release back to the driver at synchronisations), and the tile
// kernels may use large dynamic shared memory.
void device_init(int device) {
    static std::mutex mu;
    static std::vector<char> done;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= device) done.resize((size_t)device + 1, 0);
    if (done[(size_t)device]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    sc_tile_init();
    done[(size_t)device] = 1;
}

int ensure_staging(sc_sim *s, size_t bytes) {
    if (s->stagingBytes >= bytes) return SC_OK;
    if (s->staging) {
        cudaFreeAsync(s->staging, s->st);
        forget_alloc(s, (void *)s->staging);
        s->staging = nullptr;
        s->stagingBytes = 0;
    }
    int rc = dalloc(s, &s->staging, bytes);
    if (rc) return rc;
    s->stagingBytes = bytes;
    return SC_OK;
}

// The AoS staging buffer is only needed while records cross the boundary:
// it goes back to the device's pool (stream-ordered, no synchronisation)
// after each load, generation and export, which leaves a resident sim
// 304 bytes per metabolic particle lighter.
// The frame staging slots (reduced records, two per item set), allocated on
// the first frame: a sim that never reduces a frame holds none.
int ensure_frame_slots(sc_sim *s) {
    ScBuffers &B = s->B;
    if (B.redP) return SC_OK;
    const size_t N = (size_t)s->P.N, Nm = (size_t)s->P.Nm;
    int rc;
    if ((rc = dalloc(s, &B.redP, N)) || (rc = dalloc(s, &B.redM, Nm)) || (rc = dalloc(s, &B.redP2, N)) ||
        (rc = dalloc(s, &B.redM2, Nm)))
        return rc;
    return SC_OK;
}

void release_staging(sc_sim *s) {
    if (!s->staging) return;
    cudaFreeAsync(s->staging, s->st);
    forget_alloc(s, (void *)s->staging);
    s->staging = nullptr;
    s->stagingBytes = 0;
}

}  // namespace

extern "C" {

const char *sc_last_error(const sc_sim *sim) {
    if (sim) return sim->err.c_str();
    if (!g_err.empty()) return g_err.c_str();
    return sc_host_last_error();
}

static int create_sim(const sc_config *cfg_in, const sc_replica *replicas, int32_t n_replicas,
                      const sc_type_info *types, int32_t n_types, const sc_rule *rules, int32_t n_rules, sc_sim **out);

int sc_create(const sc_config *cfg, const sc_type_info *types, int32_t n_types, const sc_rule *rules, int32_t n_rules,
              sc_sim **out) {
    return create_sim(cfg, nullptr, 0, types, n_types, rules, n_rules, out);
}

int sc_create_batch(const sc_config *cfg, const sc_replica *replicas, int32_t n_replicas, const sc_type_info *types,
                    int32_t n_types, const sc_rule *rules, int32_t n_rules, sc_sim **out) {
    if (!cfg || !out || !replicas || n_replicas < 1) return set_err(nullptr, SC_E_INVALID, "bad batch arguments");
    return create_sim(cfg, replicas, n_replicas, types, n_types, rules, n_rules, out);
}

static int create_sim(const sc_config *cfg_in, const sc_replica *replicas, int32_t n_replicas,
                      const sc_type_info *types, int32_t n_types, const sc_rule *rules, int32_t n_rules, sc_sim **out) {
    if (!cfg_in || !out) return set_err(nullptr, SC_E_INVALID, "null argument");
    *out = nullptr;
    // A batch: the replicas' capacities add up, the largest box stands for the
    // sim-wide grid values; each replica's own grid is set up below.
    sc_config batchCfg = *cfg_in;
    const sc_config *cfg = cfg_in;
    if (n_replicas > 0) {
        int64_t np = 0, nmp = 0;
        float box = 0.0f;
        for (int r = 0; r < n_replicas; r++) {
            const sc_replica &q = replicas[r];
            if (q.num_particles < 0 || q.num_metabolic_particles < 0 || !(q.sim_size > 0.0f))
                return set_err(nullptr, SC_E_INVALID, "replica " + std::to_string(r) + ": bad capacity or box");
            if (cfg_in->periodic && floorf(q.sim_size / cfg_in->grid_cell_size) < 3.0f)
                return set_err(nullptr, SC_E_INVALID, "replica " + std::to_string(r) + ": a periodic box needs at least 3 grid cells per axis");
            np += q.num_particles;
            nmp += q.num_metabolic_particles;
            box = std::max(box, q.sim_size);
        }
        if (np > INT_MAX / 2 || nmp > INT_MAX / 2) return set_err(nullptr, SC_E_INVALID, "batch too large");
        for (int i = 0; i < n_rules; i++)
            if (rules && rules[i].polymerize >= 0)
                return set_err(nullptr, SC_E_INVALID, "batched sims run no polymerising rules");
        batchCfg.num_particles = (int32_t)np;
        batchCfg.num_metabolic_particles = (int32_t)nmp;
        batchCfg.sim_size = box;
        batchCfg.tiles = 0;
        cfg = &batchCfg;
    }
    if (cfg->num_particles < 0 || cfg->num_metabolic_particles < 0)
        return set_err(nullptr, SC_E_INVALID, "negative capacity");
    if (cfg->num_metabolites < 1 || cfg->num_metabolites > SC_AOS_NUM_METABOLITES)
        return set_err(nullptr, SC_E_INVALID, "num_metabolites must be in 1..10");
    if (n_types < 0 || n_rules < 0 || (n_types > 0 && !types) || (n_rules > 0 && !rules))
        return set_err(nullptr, SC_E_INVALID, "bad table arguments");
    int32_t ngrid = 0, bits = 0;
    if (sc_config_grid(cfg, &ngrid, &bits) != SC_OK) return set_err(nullptr, SC_E_INVALID, sc_host_last_error());
    if (!(cfg->max_interaction_distance >= 0.0f) || !(cfg->max_diffusion_distance >= 0.0f))
        return set_err(nullptr, SC_E_INVALID, "negative interaction distance");
    if (cfg->noise_coordination_steps < 0 || cfg->relaxation_steps < 0 || cfg->metabolite_diffusion_steps < 0)
        return set_err(nullptr, SC_E_INVALID, "negative sub-iteration count");
    // The periodic extension wraps neighbourhoods over the cells the box
    // spans; with fewer than three a cell would be visited twice.
    if (cfg->periodic && floorf(cfg->sim_size / cfg->grid_cell_size) < 3.0f)
        return set_err(nullptr, SC_E_INVALID, "a periodic box needs at least 3 grid cells per axis");

    sc_sim *s = new sc_sim();
    s->cfg = *cfg;
    if (n_types > 0) s->types.assign(types, types + n_types);
    cudaGetDevice(&s->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    s->useGraphs = cfg->graphs != 0;
    device_init(s->device);
    {
        cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copySt, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            e = cudaEventCreateWithFlags(&s->reduced[k], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->copied[k], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join[k], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            sc_destroy(s);
            return set_err(nullptr, SC_E_CUDA, cudaGetErrorString(e));
        }
    }
    s->gridCap = std::max(1, sms) * (2048 / SC_THREADS);
    ScParams &P = s->P;
    memset(&P, 0, sizeof P);
    P.simSize = cfg->sim_size;
    P.maxInt = cfg->max_interaction_distance;
    P.maxDiff = cfg->max_diffusion_distance;
    P.cell = cfg->grid_cell_size;
    P.ngrid = ngrid;
    P.bits = bits;
    P.cells = (uint32_t)ngrid * (uint32_t)ngrid * (uint32_t)ngrid;
    P.moveNoise = cfg->movement_noise_scale;
    P.rotNoise = cfg->rotation_noise_scale;
    P.metabNoise = cfg->metabolite_movement_noise_scale;
    P.velDecay = cfg->velocity_decay;
    P.angDecay = cfg->angular_velocity_decay;
    P.S = cfg->num_metabolites;
    P.SP = P.S <= 4 ? 4 : P.S <= 8 ? 8 : 12;
    P.N = cfg->num_particles;
    P.Nm = cfg->num_metabolic_particles;
    // Concurrent work classes pay off for a sim whose particles fill the
    // device; smaller sims keep one stream, so many of them run side by side
    // without the cross-stream joins (class_streams 1 / 3 overrides).
    s->forkClasses = cfg->class_streams == 0 ? (int64_t)P.N >= (int64_t)s->gridCap * SC_THREADS
                                             : cfg->class_streams > 1;
    P.coordSteps = cfg->noise_coordination_steps;
    P.seed = cfg->seed;
    // pair_list_limit >= 0 caps the pair lists (tests use it to run the
    // neighbourhood-scan path of every kernel); -1 means full capacity.
    P.listLimit = cfg->pair_list_limit >= 0 ? cfg->pair_list_limit : 1 << 30;
    P.periodic = cfg->periodic != 0;
    P.walls = cfg->walls != 0;
    P.pairClaim = cfg->pair_claim != 0;
    P.metabLean = cfg->metabolic_pairs == 0;
    P.nUsed = (int)ceilf(cfg->sim_size / cfg->grid_cell_size);
    if (cfg->periodic) P.nUsed = sc_periodic_cells(cfg->sim_size, cfg->grid_cell_size, &P.cell);
    P.nRep = 1;
    if (n_replicas > 0) {
        // Each replica's grid as a sim of its own would have it (config.cuh:65-74
        // cells per axis, or the periodic box's equal cells), its cells at
        // consecutive keys after the previous replica's; the sort orders the
        // key bits the whole key space needs.
        s->reps.assign(replicas, replicas + n_replicas);
        uint64_t base = 0;
        for (int r = 0; r < n_replicas; r++) {
            sc_config rc = *cfg;
            rc.sim_size = replicas[r].sim_size;
            int32_t ng = 0, nb = 0;
            if (sc_config_grid(&rc, &ng, &nb) != SC_OK) {
                sc_destroy(s);
                return set_err(nullptr, SC_E_INVALID, sc_host_last_error());
            }
            ScRep g;
            g.simSize = rc.sim_size;
            g.cell = rc.grid_cell_size;
            g.ngrid = ng;
            g.bits = nb;
            g.nUsed = (int)ceilf(rc.sim_size / rc.grid_cell_size);
            if (rc.periodic) g.nUsed = sc_periodic_cells(rc.sim_size, rc.grid_cell_size, &g.cell);
            g.keyBase = (uint32_t)base;
            g.seed = replicas[r].seed;
            s->repGeom.push_back(g);
            base += (uint64_t)ng * ng * ng;
        }
        if (base >= (1ull << 31)) {
            sc_destroy(s);
            return set_err(nullptr, SC_E_INVALID, "the batch's cells do not fit 31 key bits");
        }
        P.cells = (uint32_t)base;
        P.keyBits = 1;
        while ((1ull << P.keyBits) - 1 < base) P.keyBits++;
        P.nRep = n_replicas;
    }
    // Tile capacities of the metabolic sweeps from the mean occupancy of the
    // cells a tile spans, with room for fluctuations.  The tiled sweep is
    // selected with tiles = 1 (the per-item list sweep is faster at present);
    // it is off when the tile would not fit in shared memory.
    {
        const double cells = std::pow((double)std::max(P.nUsed, 1), 3.0);
        const double tileCells = (double)SC_TILE_NCOL * (SC_TILE_SZ + 3);
        auto cap = [&](double items) {
            const double mean = items / cells * tileCells;
            return (int)((1.1 * mean + 4.0 * std::sqrt(mean) + 32.0 + 31.0) / 32.0) * 32;
        };
        P.tileCapM = cap((double)P.Nm);
        P.tileCapP = cap((double)P.N);
        if (cfg->tiles != 1 || P.tileCapM + P.tileCapP > 65535 ||
            sc_tile_bytes(P.tileCapM, P.tileCapP, 32) > 200 * 1024)
            P.tileCapM = P.tileCapP = 0;
    }

    auto bail = [&](int rc) {
        sc_destroy(s);
        return rc;
    };
    // tables: id-indexed rules + zero rule, partner index, partner-mapped rules
    // (interactions.cuh:59-145; ascending rule id within a type)
    int maxId = 0;
    for (int i = 0; i < n_rules; i++) maxId = std::max(maxId, rules[i].id);
    std::vector<sc_rule> flat((size_t)maxId + 2);
    memset(flat.data(), 0, flat.size() * sizeof(sc_rule));
    std::vector<char> seen((size_t)maxId + 1, 0);
    for (int i = 0; i < n_rules; i++) {
        int id = rules[i].id;
        if (id < 0 || seen[(size_t)id]) continue;
        seen[(size_t)id] = 1;
        flat[(size_t)id] = rules[i];
        if (!cfg->rule_probabilities) {  // padding in the reference's records
            flat[(size_t)id].use_probability = 0;
            flat[(size_t)id].probability = 0.0f;
        }
    }
    std::map<int, std::vector<int>> byType;
    for (int id = 0; id <= maxId; id++) {
        if (!seen[(size_t)id]) continue;
        if (flat[(size_t)id].first_partner_type >= 0) byType[flat[(size_t)id].first_partner_type].push_back(id);
        if (flat[(size_t)id].second_partner_type >= 0) byType[flat[(size_t)id].second_partner_type].push_back(id);
    }
    std::vector<int> pidx(((size_t)maxId + 1) * 2, 0);
    std::vector<sc_rule> prules;
    for (auto &kv : byType) {
        int start = (int)prules.size();
        for (int id : kv.second) prules.push_back(flat[(size_t)id]);
        if ((size_t)kv.first * 2 + 1 < pidx.size()) {
            pidx[(size_t)kv.first * 2] = start;
            pidx[(size_t)kv.first * 2 + 1] = (int)prules.size();
        }
    }
    sc_rule *dFlat = nullptr, *dPrules = nullptr;
    int *dPidx = nullptr;
    sc_type_info *dTypes = nullptr;
    int rc;
    if ((rc = dalloc(s, &dFlat, flat.size())) || (rc = dalloc(s, &dPidx, pidx.size())) ||
        (rc = dalloc(s, &dPrules, std::max<size_t>(prules.size(), 1))) ||
        (rc = dalloc(s, &dTypes, std::max<int>(n_types, 1))))
        return bail(rc);
    // (the host vectors live until the stream is synchronised below)
    cudaMemcpyAsync(dFlat, flat.data(), flat.size() * sizeof(sc_rule), cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(dPidx, pidx.data(), pidx.size() * sizeof(int), cudaMemcpyHostToDevice, s->st);
    if (!prules.empty())
        cudaMemcpyAsync(dPrules, prules.data(), prules.size() * sizeof(sc_rule), cudaMemcpyHostToDevice, s->st);
    if (n_types > 0)
        cudaMemcpyAsync(dTypes, types, (size_t)n_types * sizeof(sc_type_info), cudaMemcpyHostToDevice, s->st);
    P.flat = dFlat;
    P.nFlat = maxId + 1;
    P.pidx = dPidx;
    P.nPidx = (int)pidx.size();
    P.prules = dPrules;
    P.types = dTypes;
    P.nTypes = n_types;
    if (!s->repGeom.empty()) {
        ScRep *dReps = nullptr;
        if ((rc = dalloc(s, &dReps, s->repGeom.size()))) return bail(rc);
        cudaMemcpyAsync(dReps, s->repGeom.data(), s->repGeom.size() * sizeof(ScRep), cudaMemcpyHostToDevice, s->st);
        P.reps = dReps;
    }

    ScBuffers &B = s->B;
    memset(&B, 0, sizeof B);
    const size_t N = (size_t)P.N, Nm = (size_t)P.Nm, Q = (size_t)P.SP / 4;
    for (int b = 0; b < 2; b++) {
        PFields &f = B.p[b];
        MFields &m = B.m[b];
        if ((rc = dalloc(s, &f.pos, N)) || (rc = dalloc(s, &f.vel, N)) || (rc = dalloc(s, &f.rot, N)) ||
            (rc = dalloc(s, &f.angvel, N)) || (rc = dalloc(s, &f.posnoise, N)) || (rc = dalloc(s, &f.angnoise, N)) ||
            (rc = dalloc(s, &f.dbg, N)) || (rc = dalloc(s, &f.info, N)) || (rc = dalloc(s, &f.state, N)) ||
            (rc = dalloc(s, &f.lscs, N)) || (rc = dalloc(s, &f.spoly, N)) || (rc = dalloc(s, &f.nb, N)) ||
            (rc = dalloc(s, &f.bonds, N * 24)) || (rc = dalloc(s, &m.vel, Nm)) || (rc = dalloc(s, &m.met, Nm * Q)) ||
            (rc = dalloc(s, &B.keysP[b], N)) || (rc = dalloc(s, &B.valsP[b], N)) || (rc = dalloc(s, &B.keysM[b], Nm)) ||
            (rc = dalloc(s, &B.valsM[b], Nm)))
            return bail(rc);
    }
    // the metabolic fields with one buffer each, and their spares
    for (int k = 0; k <= ScBuffers::kM4; k++)
        if ((rc = dalloc(s, &B.mChain4[k], Nm))) return bail(rc);
    for (int k = 0; k <= ScBuffers::kM1; k++)
        if ((rc = dalloc(s, &B.mChain1[k], Nm))) return bail(rc);
    B.setMParity(0);
    const int passes = sc_sort_passes_for(P);
    // The metabolic pair pool starts at kPoolStart entries per item (the
    // tiled sweep's 16-bit lists take the full list capacity) and sc_prepare
    // grows it to the scene's demand: a pool sized for the worst case would
    // hold most of a sim's memory.
    const int poolEntryWords = P.metabLean ? 1 : 4;
    size_t poolWords = sc_list_words(SC_LIST_M, (int)Nm);
    if (P.tileCapM == 0) poolWords = std::min(poolWords, sc_list_words(kPoolStart * poolEntryWords, (int)Nm));
    if ((rc = dalloc(s, &B.mcFlag, 4)) || (rc = dalloc(s, &B.hist, 4 * 256)) ||
        (rc = dalloc(s, &B.lookback, (size_t)passes * sc_sort_lookback_words((int)std::max(N, Nm)))) ||
        (rc = dalloc(s, &B.cellStartP, (size_t)P.cells + 1)) || (rc = dalloc(s, &B.cellStartM, (size_t)P.cells + 1)) ||
        (rc = dalloc(s, &B.polyList, N)) || (rc = dalloc(s, &B.polyRank, N)) || (rc = dalloc(s, &B.polyPmi, N)) ||
        (rc = dalloc(s, &B.polyClaim, N)) || (rc = dalloc(s, &B.polyBlk, 2 * ((size_t)N / SC_THREADS + 1))) || (rc = dalloc(s, &B.ctr, 1)) || (rc = dalloc(s, &B.listPP, sc_list_words(SC_LIST_PP, (int)N))) ||
        (rc = dalloc(s, &B.cntPP, N)) ||
        (rc = dalloc(s, &B.classPP, (size_t)SC_RELAX_CLASSES * N)) ||
        (rc = dalloc(s, &B.matchPP, (size_t)SC_MAX_ACTIVE_INTERACTIONS * N)) || (rc = dalloc(s, &B.matchN, N)) ||
        (rc = dalloc(s, &B.listM, poolWords)) ||
        (rc = dalloc(s, &B.cntM, Nm)) || (rc = dalloc(s, &B.listLM, sc_list_words(SC_LIST_LM, (int)N))) ||
        (rc = dalloc(s, &B.cntLM, N)) || (rc = dalloc(s, &B.listD, sc_list_words(SC_LIST_DBUF, (int)Nm))) ||
        (rc = dalloc(s, &B.cntD, Nm)) || (rc = dalloc(s, &B.permM, Nm)) || (rc = dalloc(s, &B.permD, Nm)) ||
        (rc = dalloc(s, &B.permLM, N)) || (rc = dalloc(s, &B.ovfPP, N)) || (rc = dalloc(s, &B.ovfM, Nm)) || (rc = dalloc(s, &B.workP, N)) ||
        (rc = dalloc(s, &B.ovfNM, Nm)) || (rc = dalloc(s, &B.ovfOffM, Nm)) || (rc = dalloc(s, &B.ovfPoolM, 1)) ||
        (rc = dalloc(s, &B.ovfD, Nm)) || (rc = dalloc(s, &B.ovfOffD, Nm)) || (rc = dalloc(s, &B.ovfPoolD, 1)) ||
        (rc = dalloc(s, &B.claimP, P.pairClaim ? N : 1)) ||
        (rc = dalloc(s, &B.warpOffM, (size_t)Nm / 32 + 1)) || (rc = dalloc(s, &B.warpOffLM, (size_t)N / 32 + 1)) ||
        (rc = dalloc(s, &B.lipidP, N)))
        return bail(rc);
    // The LM list is built in the diffusion list's buffer when it fits.
    if (sc_list_words(SC_LIST_LM, (int)N) <= sc_list_words(SC_LIST_DBUF, (int)Nm)) {
        B.scratchLM = B.listD;
    } else if ((rc = dalloc(s, &B.scratchLM, sc_list_words(SC_LIST_LM, (int)N)))) {
        return bail(rc);
    }
    B.invalidateLists();
    B.poolEntryWords = poolEntryWords;
    B.poolCapM = poolWords / B.poolEntryWords;
    // pool_per_item = n >= 0 starts the metabolic pair pool at n entries per item
    if (cfg->pool_per_item >= 0)
        B.poolCapM = std::min(B.poolCapM, (size_t)cfg->pool_per_item * (size_t)std::max<int64_t>(Nm, 1));
    P.lipidP = B.lipidP;
    cudaMemsetAsync(B.ctr, 0, sizeof(ScCounters), s->st);
    cudaMemsetAsync(B.polyClaim, 0, std::max<size_t>(N, 1) * sizeof(int), s->st);
    cudaMemsetAsync(B.cellStartP, 0, ((size_t)P.cells + 1) * 4, s->st);
    cudaMemsetAsync(B.cellStartM, 0, ((size_t)P.cells + 1) * 4, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return bail(set_err(s, SC_E_CUDA, cudaGetErrorString(e)));
    *out = s;
    return SC_OK;
}

void sc_destroy(sc_sim *s) {
    if (!s) return;
    enter(s);
    if (s->copySt) {
        cudaStreamSynchronize(s->copySt);
        cudaStreamDestroy(s->copySt);
    }
    if (s->st) {
        for (void *p : s->allocs) cudaFreeAsync(p, s->st);  // after the sim's own work
        cudaStreamSynchronize(s->st);
        cudaStreamDestroy(s->st);
    }
    for (int k = 0; k < 2; k++) {
        if (s->reduced[k]) cudaEventDestroy(s->reduced[k]);
        if (s->copied[k]) cudaEventDestroy(s->copied[k]);
        if (s->side[k]) cudaStreamDestroy(s->side[k]);  // their work is joined into st
        if (s->join[k]) cudaEventDestroy(s->join[k]);
    }
    if (s->fork) cudaEventDestroy(s->fork);
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.exec);
    delete s;
}

// The per-item copies of the metabolic fields no step kernel touches, or
// nulls when the loaded records share one value of each (B.mcUniform).
#define MC_MIRRORS(B)                                                                                      \
    ((B).mcUniform ? nullptr : (B).mcLscs), ((B).mcUniform ? nullptr : (B).mcSpoly),                     \
        ((B).mcUniform ? nullptr : (B).mcNb), ((B).mcUniform ? nullptr : (B).mcBonds)

// Decides, for the nm metabolic records now staged, whether the sim keeps
// per-item copies of the fields no step kernel touches (allocated the first
// time a load needs them) or the two values every record shares.
static int mc_prepare(sc_sim *s, int nm) {
    ScBuffers &B = s->B;
    int h[3] = {0, 0, 0};  // record 0's last state-change step and scheduled polymerisation; mixed
    if (nm > 0) {
        SC_CK(s, cudaMemsetAsync(B.mcFlag, 0, sizeof(int), s->st));
        k_mc_scan<<<nb_of(nm), SC_THREADS, 0, s->st>>>(s->staging, nm, B.mcFlag);
        SC_CK(s, cudaMemcpyAsync(&h[0], s->staging + 16, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        SC_CK(s, cudaMemcpyAsync(&h[1], s->staging + 228, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        SC_CK(s, cudaMemcpyAsync(&h[2], B.mcFlag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        SC_CK(s, cudaStreamSynchronize(s->st));
        int rc = check_launch(s);
        if (rc) return rc;
    }
    if (!h[2]) {
        B.mcUniform = true;
        B.mcLscs0 = h[0];
        B.mcSpoly0 = h[1];
        return SC_OK;
    }
    if (!B.mcLscs) {
        const size_t Nm = (size_t)s->P.Nm;
        int rc;
        if ((rc = dalloc(s, &B.mcLscs, Nm)) || (rc = dalloc(s, &B.mcSpoly, Nm)) || (rc = dalloc(s, &B.mcNb, Nm)) ||
            (rc = dalloc(s, &B.mcBonds, Nm * 24)))
            return rc;
    }
    B.mcUniform = false;
    return SC_OK;
}

// Field views from slot o on (a chunk of a load, a batch replica's slots).
static PFields shift_p(PFields f, size_t o) {
    f.pos += o; f.vel += o; f.rot += o; f.angvel += o; f.posnoise += o; f.angnoise += o; f.dbg += o; f.info += o;
    f.state += o; f.lscs += o; f.spoly += o; f.nb += o; f.bonds += 24 * o;
    return f;
}
static MFields shift_m(MFields f, size_t o, size_t q) {
    f.pos += o; f.vel += o; f.rot += o; f.angvel += o; f.posnoise += o; f.angnoise += o; f.dbg += o; f.info += o;
    f.state += o; f.met += o * q; f.orig += o;
    return f;
}

// Records cross into the device through one staging slot, a chunk at a time
// (copy, then unpack into the chunk's slots), so a load holds kStageBytes of
// staging whatever the state's size.
const size_t kStageBytes = (size_t)64 << 20;

int sc_load_state(sc_sim *s, const sc_particle *particles, int32_t n, const sc_metabolic_particle *metabolic,
                  int32_t nm, int32_t step, int32_t next_particle_id) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    const int N = s->P.N, Nm = s->P.Nm;
    if (n < 0 || nm < 0 || n > N || nm > Nm || (n > 0 && !particles) || (nm > 0 && !metabolic))
        return set_err(s, SC_E_INVALID, "state larger than the capacity or missing");
    int rc = ensure_staging(s, kStageBytes);
    if (rc) return rc;
    ScBuffers &B = s->B;
    B.invalidateLists();
    s->loaded = false;
    s->P.binned = 0;
    s->P.mAllActive = 0;
    s->P.lipidValid = 0;
    for (int k = 0; k < FP_COUNT; k++) B.cp[k] = 0;
    for (int k = 0; k < FM_COUNT; k++) B.cm[k] = 0;
    // mcFlag: [0] a metabolic record differs from the first, [1] the lowest
    // particle index with an interaction count outside 0..8
    const int flags0[2] = {0, INT_MAX};
    SC_CK(s, cudaMemcpyAsync(B.mcFlag, flags0, sizeof flags0, cudaMemcpyHostToDevice, s->st));
    const uint8_t *hp = reinterpret_cast<const uint8_t *>(particles);
    const int perP = (int)(kStageBytes / sizeof(sc_particle));
    for (int i0 = 0; i0 < n; i0 += perP) {
        const int cnt = std::min(perP, n - i0);
        SC_CK(s, cudaMemcpyAsync(s->staging, hp + (size_t)i0 * sizeof(sc_particle), (size_t)cnt * sizeof(sc_particle),
                                 cudaMemcpyHostToDevice, s->st));
        k_unpack_particles<<<nb_of(cnt), SC_THREADS, 0, s->st>>>(s->staging, cnt, cnt, shift_p(B.p[0], (size_t)i0),
                                                                 B.mcFlag + 1, i0);
    }
    if (N > n)
        k_unpack_particles<<<nb_of(N - n), SC_THREADS, 0, s->st>>>(s->staging, 0, N - n, shift_p(B.p[0], (size_t)n));
    // metabolic records: unpacked as sharing one value of each untouched field
    // (every scene here), scanned as they pass; a load that turns out mixed
    // is unpacked again with per-item copies
    const uint8_t *hm = reinterpret_cast<const uint8_t *>(metabolic);
    const int lscs0 = nm > 0 ? metabolic[0].p.last_state_change_step : 0;
    const int spoly0 = nm > 0 ? metabolic[0].p.scheduled_polymerization : 0;
    const int perM = (int)(kStageBytes / sizeof(sc_metabolic_particle));
    const size_t Q = (size_t)s->P.SP / 4;
    for (int pass = 0; pass < 2; pass++) {
        const bool mirrors = pass == 1;
        for (int i0 = 0; i0 < nm; i0 += perM) {
            const int cnt = std::min(perM, nm - i0);
            SC_CK(s, cudaMemcpyAsync(s->staging, hm + (size_t)i0 * sizeof(sc_metabolic_particle),
                                     (size_t)cnt * sizeof(sc_metabolic_particle), cudaMemcpyHostToDevice, s->st));
            if (!mirrors)
                k_mc_scan_ref<<<nb_of(cnt), SC_THREADS, 0, s->st>>>(s->staging, cnt, lscs0, spoly0, B.mcFlag);
            k_unpack_metabolic<<<nb_of(cnt), SC_THREADS, 0, s->st>>>(
                s->staging, cnt, cnt, s->P.SP, shift_m(B.m[0], (size_t)i0, Q), mirrors ? B.mcLscs + i0 : nullptr,
                mirrors ? B.mcSpoly + i0 : nullptr, mirrors ? B.mcNb + i0 : nullptr,
                mirrors ? B.mcBonds + (size_t)i0 * 24 : nullptr, i0);
        }
        if (Nm > nm)
            k_unpack_metabolic<<<nb_of(Nm - nm), SC_THREADS, 0, s->st>>>(
                s->staging, 0, Nm - nm, s->P.SP, shift_m(B.m[0], (size_t)nm, Q), mirrors ? B.mcLscs + nm : nullptr,
                mirrors ? B.mcSpoly + nm : nullptr, mirrors ? B.mcNb + nm : nullptr,
                mirrors ? B.mcBonds + (size_t)nm * 24 : nullptr, nm);
        int flags[2] = {0, INT_MAX};
        SC_CK(s, cudaMemcpyAsync(flags, B.mcFlag, sizeof flags, cudaMemcpyDeviceToHost, s->st));
        SC_CK(s, cudaStreamSynchronize(s->st));
        if ((rc = check_launch(s))) return rc;
        if (flags[1] != INT_MAX)
            return set_err(s, SC_E_INVALID, "particle " + std::to_string(flags[1]) + " has more than 8 interactions");
        if (mirrors || !flags[0]) {
            B.mcUniform = !mirrors;
            B.mcLscs0 = lscs0;
            B.mcSpoly0 = spoly0;
            break;
        }
        if (!B.mcLscs && ((rc = dalloc(s, &B.mcLscs, (size_t)Nm)) || (rc = dalloc(s, &B.mcSpoly, (size_t)Nm)) ||
                          (rc = dalloc(s, &B.mcNb, (size_t)Nm)) || (rc = dalloc(s, &B.mcBonds, (size_t)Nm * 24))))
            return rc;
    }
    ScCounters c;
    memset(&c, 0, sizeof c);
    c.nActive = n;
    c.lastActive = n - 1;
    c.nextId = next_particle_id;
    c.nActiveM = nm;
    c.step = step;
    SC_CK(s, cudaMemcpyAsync(B.ctr, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    rc = check_launch(s);
    if (rc) return rc;
    release_staging(s);
    s->loaded = true;
    return SC_OK;
}

static int grow_pools(sc_sim *s);

int sc_prepare(sc_sim *s) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    enter(s);
    int rc;
    if ((rc = run_phase(s, SC_PHASE_SORT_PARTICLES, 0)) || (rc = run_phase(s, SC_PHASE_SORT_METABOLIC, 0)) ||
        (rc = run_phase(s, SC_PHASE_REMOVE_INTERFERING, 0)) || (rc = run_phase(s, SC_PHASE_COMPLEXIFY, -1)))
        return rc;
    // the metabolic pair pool sized for this scene: its list built once,
    // its demand read back, the pool grown to it (1.25x); a pool whose
    // starting size the config fixes (pool_per_item >= 0) is left to grow at
    // the next synchronisation
    if (s->cfg.pool_per_item >= 0) return SC_OK;
    ScLaunchCtx c = ctx(s);
    sc_phase_build_m(c);
    if ((rc = check_launch(s))) return rc;
    SC_CK(s, cudaStreamSynchronize(s->st));
    return grow_pools(s);
}

int sc_run_phase(sc_sim *s, int32_t phase, int32_t arg) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    enter(s);
    return run_phase(s, phase, arg);
}

int sc_step(sc_sim *s, int32_t n_steps) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    if (n_steps < 0) return set_err(s, SC_E_INVALID, "negative step count");
    enter(s);
    for (int k = 0; k < n_steps; k++) {
        int rc = s->useGraphs ? step_graph(s) : step_direct(s);
        if (rc) return rc;
    }
    if (s->notifyKey >= 0) SC_CK(s, cudaLaunchHostFunc(s->st, notice_cb, (void *)(intptr_t)s->notifyKey));
    return SC_OK;
}

int sc_set_notify(sc_sim *s, int64_t key) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    s->notifyKey = key < 0 ? -1 : key;
    return SC_OK;
}

int32_t sc_wait_notices(int64_t *keys, int32_t cap, int32_t timeout_ms) {
    if (!keys || cap < 1) return set_err(nullptr, SC_E_INVALID, "no room for notices");
    std::unique_lock<std::mutex> lk(g_noticeMu);
    if (g_notices.empty() && timeout_ms != 0) {
        auto ready = [] { return !g_notices.empty(); };
        if (timeout_ms < 0) g_noticeCv.wait(lk, ready);
        else g_noticeCv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
    }
    int32_t n = 0;
    while (n < cap && !g_notices.empty()) {
        keys[n++] = g_notices.front();
        g_notices.pop_front();
    }
    return n;
}


// The metabolic pair pool is sized for the lists the sim needs: its last
// build's demand (what every block asked for, granted or not) is read at
// each synchronisation and, when it exceeded the pool, the pool grows to
// 1.25x the demand.  Lists of blocks the pool had no room for were scanned
// instead, so results never depend on the pool's size; step graphs, which
// hold the old buffer, are dropped.  Called with the sim's streams idle.
// An overflow pool (the overflowed metabolic items', or the diffusion
// lists') grown to its last demand (1.25x), the old one released first;
// without room it keeps its old size.  Growing drops the lists and the step
// graphs, which hold the old buffer.
extern "C++" template <class T>
int grow_ovf_pool(sc_sim *s, const unsigned long long *demand, T *&pool, size_t &capacity) {
    ScBuffers &B = s->B;
    unsigned long long need = 0;
    SC_CK(s, cudaMemcpy(&need, demand, sizeof need, cudaMemcpyDeviceToHost));
    if (need <= capacity) return SC_OK;
    const size_t cap = (size_t)need + (size_t)need / 4 + 1024;
    forget_alloc(s, (void *)pool);
    SC_CK(s, cudaFreeAsync(pool, s->st));
    pool = nullptr;
    B.validM = B.validD = false;
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.exec);
    s->graphs.clear();
    int rc = dalloc(s, &pool, cap);
    if (rc) {
        s->err.clear();
        return dalloc(s, &pool, std::max<size_t>(capacity, 1));
    }
    capacity = cap;
    return SC_OK;
}

// The main metabolic pool first: when it had no room, whole blocks of
// ordinary lists overflowed into the overflow pool (at 16 bytes a pair), so
// that pool's demand is only taken at a synchronisation where the main pool
// did not grow.
static int grow_main_pool(sc_sim *s, bool *grew);
static int grow_pools(sc_sim *s) {
    ScBuffers &B = s->B;
    bool grew = false;
    int rc;
    if ((rc = grow_main_pool(s, &grew))) return rc;
    if (!grew && (rc = grow_ovf_pool(s, &B.ctr->poolOvfM, B.ovfPoolM, B.ovfPoolCapM))) return rc;
    return grow_ovf_pool(s, &B.ctr->poolOvfD, B.ovfPoolD, B.ovfPoolCapD);
}

static int grow_main_pool(sc_sim *s, bool *grew) {
    ScBuffers &B = s->B;
    unsigned long long need = 0;
    SC_CK(s, cudaMemcpy(&need, &B.ctr->poolM, sizeof need, cudaMemcpyDeviceToHost));
    if (need <= B.poolCapM) return SC_OK;
    const size_t cap = (size_t)need + (size_t)need / 4 + 1024;
    // the old pool goes back to the device's pool first (its lists are
    // rebuilt anyway), so the new one can take its memory
    const size_t old = B.poolCapM;
    forget_alloc(s, (void *)B.listM);
    SC_CK(s, cudaFreeAsync(B.listM, s->st));
    B.listM = nullptr;
    B.validM = false;
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.exec);  // they hold the old buffer
    s->graphs.clear();
    uint32_t *grown = nullptr;
    int rc = dalloc(s, &grown, cap * B.poolEntryWords);
    if (rc) {  // no room: a pool of the old size again (the overflowing blocks keep scanning)
        s->err.clear();
        if ((rc = dalloc(s, &grown, old * B.poolEntryWords))) return rc;
        B.listM = grown;
        return SC_OK;
    }
    B.listM = grown;
    B.poolCapM = cap;
    *grew = true;
    return SC_OK;
}

int sc_sync(sc_sim *s) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    SC_CK(s, cudaStreamSynchronize(s->st));
    SC_CK(s, cudaStreamSynchronize(s->copySt));
    int derr = 0;
    SC_CK(s, cudaMemcpy(&derr, &s->B.ctr->error, sizeof(int), cudaMemcpyDeviceToHost));
    if (derr) return set_err(s, SC_E_DEVICE, "device-side error code " + std::to_string(derr));
    return s->loaded ? grow_pools(s) : SC_OK;
}

int sc_pair_counts(sc_sim *s, int64_t out[4]) {
    if (!s || !out) return set_err(s, SC_E_INVALID, "null argument");
    enter(s);
    const ScBuffers &B = s->B;
    const int *cnt[4] = {B.cntPP, B.cntM, B.cntLM, B.cntD};
    const bool valid[4] = {B.validPP, B.validM, B.validLM, B.validD};
    const int cap[4] = {s->P.N, s->P.Nm, s->P.N, s->P.Nm};
    const int *nact[4] = {&B.ctr->nActive, &B.ctr->nActiveM, &B.ctr->nActive, &B.ctr->nActiveM};
    long long *d = nullptr;
    SC_CK(s, cudaMallocAsync((void **)&d, 4 * sizeof(long long), s->st));
    SC_CK(s, cudaMemsetAsync(d, 0, 4 * sizeof(long long), s->st));
    for (int k = 0; k < 4; k++)
        if (valid[k] && cap[k] > 0)
            k_sum_counts<<<std::max(1, std::min(nb_of(cap[k]), 1024)), SC_THREADS, 0, s->st>>>(cnt[k], nact[k], d + k);
    long long h[4] = {0, 0, 0, 0};
    SC_CK(s, cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s->st));
    SC_CK(s, cudaFreeAsync(d, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    for (int k = 0; k < 4; k++) out[k] = valid[k] ? (int64_t)h[k] : -1;
    return check_launch(s);
}

int sc_list_overflows(sc_sim *s, int64_t out[4]) {
    if (!s || !out) return set_err(s, SC_E_INVALID, "null argument");
    enter(s);
    const ScBuffers &B = s->B;
    const int *cnt[4] = {B.cntPP, B.cntM, B.cntLM, B.cntD};
    const bool valid[4] = {B.validPP, B.validM, B.validLM, B.validD};
    const int cap[4] = {s->P.N, s->P.Nm, s->P.N, s->P.Nm};
    const int lim = s->P.listLimit;
    const int limit[4] = {std::min(SC_LIST_PP, lim), std::min(SC_LIST_M, lim), std::min(SC_LIST_LM, lim),
                          std::min(SC_LIST_D, lim)};
    const int *nact[4] = {&B.ctr->nActive, &B.ctr->nActiveM, &B.ctr->nActive, &B.ctr->nActiveM};
    long long *d = nullptr;
    SC_CK(s, cudaMallocAsync((void **)&d, 4 * sizeof(long long), s->st));
    SC_CK(s, cudaMemsetAsync(d, 0, 4 * sizeof(long long), s->st));
    for (int k = 0; k < 4; k++)
        if (valid[k] && cap[k] > 0)
            k_count_over<<<std::max(1, std::min(nb_of(cap[k]), 1024)), SC_THREADS, 0, s->st>>>(cnt[k], nact[k],
                                                                                            limit[k], d + k);
    long long h[4] = {0, 0, 0, 0};
    SC_CK(s, cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s->st));
    SC_CK(s, cudaFreeAsync(d, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    for (int k = 0; k < 4; k++) out[k] = valid[k] ? (int64_t)h[k] : -1;
    return check_launch(s);
}

int sc_idle(sc_sim *s) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    for (cudaStream_t st : {s->st, s->copySt}) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaErrorNotReady) return 0;
        if (e != cudaSuccess) return set_err(s, SC_E_CUDA, cudaGetErrorString(e));
    }
    return 1;
}

int sc_get_counters(sc_sim *s, sc_counters *out) {
    if (!s || !out) return set_err(s, SC_E_INVALID, "null argument");
    int rc = sc_sync(s);
    ScCounters c;
    SC_CK(s, cudaMemcpy(&c, s->B.ctr, sizeof c, cudaMemcpyDeviceToHost));
    memset(out, 0, sizeof *out);
    out->n_active_particles = c.nActive;
    out->n_active_metabolic_particles = c.nActiveM;
    out->next_particle_id = c.nextId;
    out->step = c.step;
    out->kernel_launches = s->launches;
    out->device_error = c.error;
    return rc == SC_E_DEVICE ? SC_OK : rc;
}

void *sc_get_stream(sc_sim *s) { return s ? (void *)s->st : nullptr; }

int sc_device_bytes(const sc_sim *s, int64_t *bytes) {
    if (!s || !bytes) return set_err(nullptr, SC_E_INVALID, "null argument");
    int64_t t = 0;
    for (const auto &kv : s->allocBytes) t += (int64_t)kv.second;
    *bytes = t;
    return SC_OK;
}

// The records of slots [0, cap) of one item set, packed chunk by chunk
// through the staging slot (kStageBytes at most, whatever the state's size):
// take(first slot, count) runs once a chunk's records are in the slot.
static int staged_pack(sc_sim *s, bool metabolic, const std::function<int(int, int)> &take) {
    const int cap = metabolic ? s->P.Nm : s->P.N;
    if (cap <= 0) return SC_OK;
    const size_t rec = metabolic ? sizeof(sc_metabolic_particle) : sizeof(sc_particle);
    const int chunk = (int)std::min<size_t>((size_t)cap, kStageBytes / rec);
    int rc = ensure_staging(s, (size_t)chunk * rec);
    if (rc) return rc;
    ScBuffers &B = s->B;
    for (int base = 0; base < cap; base += chunk) {
        const int end = (int)std::min<long long>((long long)base + chunk, cap);
        if (metabolic)
            k_pack_metabolic<<<nb_of(end - base), SC_THREADS, 0, s->st>>>(s->staging, &B.ctr->nActiveM, base, end,
                                                                          s->P.SP, B.M(), MC_MIRRORS(B), B.mcLscs0,
                                                                          B.mcSpoly0);
        else
            k_pack_particles<<<nb_of(end - base), SC_THREADS, 0, s->st>>>(s->staging, &B.ctr->nActive, base, end,
                                                                          B.P());
        SC_CK(s, cudaStreamSynchronize(s->st));
        if ((rc = check_launch(s)) || (rc = take(base, end - base))) return rc;
    }
    return SC_OK;
}

int sc_export_state(sc_sim *s, sc_particle *particles, sc_metabolic_particle *metabolic) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    SC_CK(s, cudaStreamSynchronize(s->st));
    int rc = SC_OK;
    if (particles)
        rc = staged_pack(s, false, [&](int first, int count) {
            SC_CK(s, cudaMemcpy(particles + first, s->staging, (size_t)count * sizeof(sc_particle),
                                cudaMemcpyDeviceToHost));
            return SC_OK;
        });
    if (!rc && metabolic)
        rc = staged_pack(s, true, [&](int first, int count) {
            SC_CK(s, cudaMemcpy(metabolic + first, s->staging, (size_t)count * sizeof(sc_metabolic_particle),
                                cudaMemcpyDeviceToHost));
            return SC_OK;
        });
    release_staging(s);
    return rc ? rc : check_launch(s);
}

static int set_batch_reps(sc_sim *s, const std::vector<int> &offP, const std::vector<int> &offM);

int sc_load_batch(sc_sim *s, const sc_particle *particles, const int32_t *n, const sc_metabolic_particle *metabolic,
                  const int32_t *nm, int32_t step) {
    if (!s || !n || !nm) return set_err(s, SC_E_INVALID, "null argument");
    if (s->reps.empty()) return set_err(s, SC_E_STATE, "not a batched sim");
    const int R = (int)s->reps.size();
    std::vector<int> offP(R + 1, 0), offM(R + 1, 0);
    for (int r = 0; r < R; r++) {
        if (n[r] < 0 || nm[r] < 0 || n[r] > s->reps[r].num_particles || nm[r] > s->reps[r].num_metabolic_particles)
            return set_err(s, SC_E_INVALID, "replica " + std::to_string(r) + ": state larger than its capacity");
        offP[r + 1] = offP[r] + n[r];
        offM[r + 1] = offM[r] + nm[r];
    }
    int rc = sc_load_state(s, particles, offP[R], metabolic, offM[R], step, 0);
    if (rc) return rc;
    return set_batch_reps(s, offP, offM);
}

// The replica ids of a batch just loaded or generated, from the replicas'
// item counts (offsets: prefix sums).
static int set_batch_reps(sc_sim *s, const std::vector<int> &offP, const std::vector<int> &offM) {
    const int R = (int)s->reps.size();
    int rc;
    int *dOff = nullptr;
    if ((rc = dalloc(s, &dOff, 2 * ((size_t)R + 1)))) return rc;
    SC_CK(s, cudaMemcpyAsync(dOff, offP.data(), (R + 1) * sizeof(int), cudaMemcpyHostToDevice, s->st));
    SC_CK(s, cudaMemcpyAsync(dOff + R + 1, offM.data(), (R + 1) * sizeof(int), cudaMemcpyHostToDevice, s->st));
    ScBuffers &B = s->B;
    if (s->P.N > 0) k_set_reps<<<nb_of(s->P.N), SC_THREADS, 0, s->st>>>(B.p[0].info, s->P.N, dOff, R);
    if (s->P.Nm > 0) k_set_reps<<<nb_of(s->P.Nm), SC_THREADS, 0, s->st>>>(B.m[0].info, s->P.Nm, dOff + R + 1, R);
    SC_CK(s, cudaStreamSynchronize(s->st));
    cudaFreeAsync(dOff, s->st);
    forget_alloc(s, (void *)dOff);
    return check_launch(s);
}

// The slots of replica r in slot order (from the info records' replica bits).
static int replica_slots(sc_sim *s, const int4 *info, int cap, int r, std::vector<std::pair<int, int>> &runs) {
    std::vector<int4> h((size_t)std::max(cap, 1));
    if (cap > 0) SC_CK(s, cudaMemcpy(h.data(), info, (size_t)cap * sizeof(int4), cudaMemcpyDeviceToHost));
    runs.clear();
    for (int i = 0; i < cap; i++) {
        if ((int)((unsigned)h[(size_t)i].w >> 8) != r) continue;
        if (!runs.empty() && runs.back().first + runs.back().second == i) runs.back().second++;
        else runs.push_back({i, 1});
    }
    return SC_OK;
}

// Replica r's records of one item set: its slots' runs (slot order) packed
// chunk by chunk, each run's part in a chunk copied to its place in `out`
// (cap records at most; the rest of `out` zero).
static int export_replica_set(sc_sim *s, int r, bool metabolic, uint8_t *out, size_t cap) {
    const size_t rec = metabolic ? sizeof(sc_metabolic_particle) : sizeof(sc_particle);
    memset(out, 0, cap * rec);
    const int n = metabolic ? s->P.Nm : s->P.N;
    if (n <= 0) return SC_OK;
    std::vector<std::pair<int, int>> runs;
    int rc = replica_slots(s, metabolic ? s->B.M().info : s->B.P().info, n, r, runs);
    if (rc) return rc;
    // output position of each run
    std::vector<size_t> at(runs.size());
    size_t k = 0;
    for (size_t u = 0; u < runs.size(); u++) {
        at[u] = k;
        k += (size_t)runs[u].second;
    }
    size_t u0 = 0;  // first run not yet wholly before the chunk
    return staged_pack(s, metabolic, [&](int first, int count) {
        const int last = first + count;
        while (u0 < runs.size() && runs[u0].first + runs[u0].second <= first) u0++;
        for (size_t u = u0; u < runs.size() && runs[u].first < last; u++) {
            const int lo = std::max(first, runs[u].first), hi = std::min(last, runs[u].first + runs[u].second);
            const size_t dst = at[u] + (size_t)(lo - runs[u].first);
            if (hi <= lo || dst >= cap) continue;
            const size_t m = std::min((size_t)(hi - lo), cap - dst);
            SC_CK(s, cudaMemcpy(out + dst * rec, s->staging + (size_t)(lo - first) * rec, m * rec,
                                cudaMemcpyDeviceToHost));
        }
        return SC_OK;
    });
}

int sc_export_replica(sc_sim *s, int32_t r, sc_particle *particles, sc_metabolic_particle *metabolic) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (s->reps.empty()) return set_err(s, SC_E_STATE, "not a batched sim");
    if (r < 0 || r >= (int)s->reps.size()) return set_err(s, SC_E_INVALID, "no such replica");
    enter(s);
    SC_CK(s, cudaStreamSynchronize(s->st));
    int rc = SC_OK;
    if (particles)
        rc = export_replica_set(s, r, false, reinterpret_cast<uint8_t *>(particles),
                                (size_t)s->reps[(size_t)r].num_particles);
    if (!rc && metabolic)
        rc = export_replica_set(s, r, true, reinterpret_cast<uint8_t *>(metabolic),
                                (size_t)s->reps[(size_t)r].num_metabolic_particles);
    release_staging(s);
    return rc ? rc : check_launch(s);
}

int sc_export_grid(sc_sim *s, int32_t which, uint32_t *ranges, uint32_t *perm) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    SC_CK(s, cudaStreamSynchronize(s->st));
    const uint32_t cells = s->P.cells;
    const int cap = which ? s->P.Nm : s->P.N;
    if (ranges) {
        std::vector<uint32_t> cs((size_t)cells + 1);
        SC_CK(s, cudaMemcpy(cs.data(), which ? s->B.cellStartM : s->B.cellStartP, cs.size() * 4, cudaMemcpyDeviceToHost));
        for (uint32_t c = 0; c < cells; c++) {
            bool empty = cs[c] == cs[c + 1];
            ranges[2 * (size_t)c] = empty ? 0 : cs[c];
            ranges[2 * (size_t)c + 1] = empty ? 0 : cs[c + 1];
        }
    }
    if (perm && cap > 0) {
        const uint32_t *src = which ? s->B.valsM[s->B.sortCurM] : s->B.valsP[s->B.sortCurP];
        SC_CK(s, cudaMemcpy(perm, src, (size_t)cap * 4, cudaMemcpyDeviceToHost));
    }
    return SC_OK;
}

int sc_reduce_frame(sc_sim *s, sc_reduced_particle *particles, sc_reduced_metabolic_particle *metabolic) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    int rc = ensure_frame_slots(s);
    if (rc) return rc;
    ScLaunchCtx c = ctx(s);
    // the synchronous form uses slot 0 once the frames in flight have landed
    if (s->frames > 0) SC_CK(s, cudaStreamSynchronize(s->copySt));
    sc_phase_reduce(c, 0);
    rc = check_launch(s);
    if (rc) return rc;
    if (particles && s->P.N > 0)
        SC_CK(s, cudaMemcpyAsync(particles, s->B.redP, (size_t)s->P.N * sizeof(sc_reduced_particle),
                                 cudaMemcpyDeviceToHost, s->st));
    if (metabolic && s->P.Nm > 0)
        SC_CK(s, cudaMemcpyAsync(metabolic, s->B.redM, (size_t)s->P.Nm * sizeof(sc_reduced_metabolic_particle),
                                 cudaMemcpyDeviceToHost, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    return SC_OK;
}

// The common part of the scene generators: resets the host-side state,
// runs `particles` (which writes the n particle records into the staging
// buffer on the sim's stream), unpacks them, generates and unpacks nm
// metabolic particles and sets the counters.
static int generate_into(sc_sim *s, int n, int nm, uint64_t seed, const std::function<void(float)> &particles) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    const int N = s->P.N, Nm = s->P.Nm;
    if (nm > 0 && (int)s->types.size() <= SC_PARTICLE_TYPE_METABOLIC)
        return set_err(s, SC_E_INVALID, "the type table has no metabolic particle type (1000)");
    size_t bytes = std::max((size_t)n * sizeof(sc_particle), (size_t)nm * sizeof(sc_metabolic_particle));
    int rc = ensure_staging(s, std::max<size_t>(bytes, 16));
    if (rc) return rc;
    ScBuffers &B = s->B;
    B.invalidateLists();
    s->P.binned = 0;
    s->P.mAllActive = 0;
    s->P.lipidValid = 0;
    for (int k = 0; k < FP_COUNT; k++) B.cp[k] = 0;
    for (int k = 0; k < FM_COUNT; k++) B.cm[k] = 0;
    const float box = s->cfg.sim_size;
    if (N > 0) {
        if (n) particles(box);
        k_unpack_particles<<<nb_of(N), SC_THREADS, 0, s->st>>>(s->staging, n, N, B.p[0]);
    }
    if (Nm > 0) {
        if (nm) {
            const sc_type_info &mt = s->types[SC_PARTICLE_TYPE_METABOLIC];
            k_gen_metabolic<<<nb_of(nm), SC_THREADS, 0, s->st>>>(s->staging, nm, box, s->cfg.num_metabolites,
                                                                 mt.radius, mt.hydrophobic, seed);
        }
        if ((rc = mc_prepare(s, nm))) return rc;
        k_unpack_metabolic<<<nb_of(Nm), SC_THREADS, 0, s->st>>>(s->staging, nm, Nm, s->P.SP, B.m[0], MC_MIRRORS(B));
    }
    ScCounters c;
    memset(&c, 0, sizeof c);
    c.nActive = n;
    c.lastActive = n - 1;
    c.nextId = n;
    c.nActiveM = nm;
    SC_CK(s, cudaMemcpyAsync(B.ctr, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    rc = check_launch(s);
    if (rc) return rc;
    release_staging(s);
    s->loaded = true;
    return SC_OK;
}

int sc_generate_uniform(sc_sim *s, int32_t n, int32_t nm, const int32_t *kinds, const float *fractions,
                        int32_t nkinds, uint64_t seed) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    if (n < 0 || nm < 0 || n > s->P.N || nm > s->P.Nm) return set_err(s, SC_E_INVALID, "scene larger than the capacity");
    sc_gen_mix mix;
    memset(&mix, 0, sizeof mix);
    if (n > 0 && (!kinds || !fractions ||
                  sc_gen_make_mix(&mix, kinds, fractions, nkinds, s->types.data(), (int)s->types.size())))
        return set_err(s, SC_E_INVALID, "the particle mix needs 1 to 4 kinds of the type table, weights >= 0");
    return generate_into(s, n, nm, seed, [&](float box) {
        k_gen_particles<<<nb_of(n), SC_THREADS, 0, s->st>>>(s->staging, n, box, mix, seed);
    });
}

int sc_generate_batch(sc_sim *s, const int32_t *n, const int32_t *nm, const int32_t *kinds, const float *fractions,
                      int32_t nkinds, const uint64_t *seeds) {
    if (!s || !n || !nm || !seeds) return set_err(s, SC_E_INVALID, "null argument");
    if (s->reps.empty()) return set_err(s, SC_E_STATE, "not a batched sim");
    enter(s);
    const int R = (int)s->reps.size();
    std::vector<int> offP(R + 1, 0), offM(R + 1, 0);
    std::vector<sc_gen_mix> mix((size_t)R);
    for (int r = 0; r < R; r++) {
        if (n[r] < 0 || nm[r] < 0 || n[r] > s->reps[r].num_particles || nm[r] > s->reps[r].num_metabolic_particles)
            return set_err(s, SC_E_INVALID, "replica " + std::to_string(r) + ": scene larger than its capacity");
        memset(&mix[r], 0, sizeof mix[r]);
        if (n[r] > 0 && (!kinds || !fractions ||
                         sc_gen_make_mix(&mix[r], kinds, fractions + (size_t)r * nkinds, nkinds, s->types.data(),
                                         (int)s->types.size())))
            return set_err(s, SC_E_INVALID, "the particle mix needs 1 to 4 kinds of the type table, weights >= 0");
        offP[r + 1] = offP[r] + n[r];
        offM[r + 1] = offM[r] + nm[r];
    }
    if (offM[R] > 0 && (int)s->types.size() <= SC_PARTICLE_TYPE_METABOLIC)
        return set_err(s, SC_E_INVALID, "the type table has no metabolic particle type (1000)");
    const int N = s->P.N, Nm = s->P.Nm;
    size_t bytes = std::max((size_t)offP[R] * sizeof(sc_particle), (size_t)offM[R] * sizeof(sc_metabolic_particle));
    int rc = ensure_staging(s, std::max<size_t>(bytes, 16));
    if (rc) return rc;
    ScBuffers &B = s->B;
    B.invalidateLists();
    s->P.binned = 0;
    s->P.mAllActive = 0;
    s->P.lipidValid = 0;
    for (int k = 0; k < FP_COUNT; k++) B.cp[k] = 0;
    for (int k = 0; k < FM_COUNT; k++) B.cm[k] = 0;
    // each replica's records as sc_generate_uniform writes them for a sim of
    // its own (ids from 0, its box, its mix and seed), one replica after another
    if (N > 0) {
        for (int r = 0; r < R; r++)
            if (n[r] > 0)
                k_gen_particles<<<nb_of(n[r]), SC_THREADS, 0, s->st>>>(
                    s->staging + (size_t)offP[r] * sizeof(sc_particle), n[r], s->reps[r].sim_size, mix[r], seeds[r]);
        k_unpack_particles<<<nb_of(N), SC_THREADS, 0, s->st>>>(s->staging, offP[R], N, B.p[0]);
    }
    if (Nm > 0) {
        const sc_type_info &mt = s->types[SC_PARTICLE_TYPE_METABOLIC];
        for (int r = 0; r < R; r++)
            if (nm[r] > 0)
                k_gen_metabolic<<<nb_of(nm[r]), SC_THREADS, 0, s->st>>>(
                    s->staging + (size_t)offM[r] * sizeof(sc_metabolic_particle), nm[r], s->reps[r].sim_size,
                    s->cfg.num_metabolites, mt.radius, mt.hydrophobic, seeds[r]);
        if ((rc = mc_prepare(s, offM[R]))) return rc;
        k_unpack_metabolic<<<nb_of(Nm), SC_THREADS, 0, s->st>>>(s->staging, offM[R], Nm, s->P.SP, B.m[0], MC_MIRRORS(B));
    }
    ScCounters c;
    memset(&c, 0, sizeof c);
    c.nActive = offP[R];
    c.lastActive = offP[R] - 1;
    c.nActiveM = offM[R];
    SC_CK(s, cudaMemcpyAsync(B.ctr, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    if ((rc = check_launch(s))) return rc;
    release_staging(s);
    s->loaded = true;
    return set_batch_reps(s, offP, offM);
}

int sc_generate_scene(sc_sim *s, const sc_scene_group *groups, int32_t n_groups, int32_t nm, uint64_t seed) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    if (n_groups < 0 || (n_groups > 0 && !groups) || nm < 0 || nm > s->P.Nm)
        return set_err(s, SC_E_INVALID, "bad group list or metabolic count");
    std::vector<sc_gen_group> gg((size_t)std::max(n_groups, 1));
    const char *why = "";
    const int64_t total = sc_gen_prepare(groups, n_groups, s->types.data(), (int32_t)s->types.size(), gg.data(), &why);
    if (total < 0) return set_err(s, SC_E_INVALID, why);
    const int n = (int)total;
    if (n > s->P.N) return set_err(s, SC_E_INVALID, "scene larger than the capacity");
    return generate_into(s, n, nm, seed, [&](float box) {
        for (int32_t g = 0; g < n_groups; g++) {
            const sc_gen_group &G = gg[(size_t)g];
            const int per = (G.kind == SC_SCENE_COMPLEXES || G.kind == SC_SCENE_WRAPPED_CHAINS) ? G.unit : 1;
            if (G.count > 0)
                k_gen_scene<<<nb_of(G.count), SC_THREADS, 0, s->st>>>(s->staging, G, per, box, seed);
        }
    });
}

int sc_generate_scene_batch(sc_sim *s, const sc_scene_group *groups, int32_t n_groups, int32_t nm,
                            const uint64_t *seeds) {
    if (!s || !seeds) return set_err(s, SC_E_INVALID, "null argument");
    if (s->reps.empty()) return set_err(s, SC_E_STATE, "not a batched sim");
    enter(s);
    const int R = (int)s->reps.size();
    if (n_groups < 0 || (n_groups > 0 && !groups) || nm < 0) return set_err(s, SC_E_INVALID, "bad group list");
    std::vector<sc_gen_group> gg((size_t)std::max(n_groups, 1));
    const char *why = "";
    const int64_t total = sc_gen_prepare(groups, n_groups, s->types.data(), (int32_t)s->types.size(), gg.data(), &why);
    if (total < 0) return set_err(s, SC_E_INVALID, why);
    const int n = (int)total;
    std::vector<int> offP(R + 1, 0), offM(R + 1, 0);
    for (int r = 0; r < R; r++) {
        if (n > s->reps[r].num_particles || nm > s->reps[r].num_metabolic_particles)
            return set_err(s, SC_E_INVALID, "replica " + std::to_string(r) + ": scene larger than its capacity");
        offP[r + 1] = offP[r] + n;
        offM[r + 1] = offM[r] + nm;
    }
    if (nm > 0 && (int)s->types.size() <= SC_PARTICLE_TYPE_METABOLIC)
        return set_err(s, SC_E_INVALID, "the type table has no metabolic particle type (1000)");
    const int N = s->P.N, Nm = s->P.Nm;
    int rc = ensure_staging(s, std::max<size_t>(std::max((size_t)n * sizeof(sc_particle),
                                                         (size_t)nm * sizeof(sc_metabolic_particle)), 16));
    if (rc) return rc;
    ScBuffers &B = s->B;
    B.invalidateLists();
    s->P.binned = 0;
    s->P.mAllActive = 0;
    s->P.lipidValid = 0;
    for (int k = 0; k < FP_COUNT; k++) B.cp[k] = 0;
    for (int k = 0; k < FM_COUNT; k++) B.cm[k] = 0;
    const size_t Q = (size_t)s->P.SP / 4;
    const sc_type_info *mt = nm > 0 ? &s->types[SC_PARTICLE_TYPE_METABOLIC] : nullptr;
    bool uniform = true;
    int lscs0 = 0, spoly0 = 0;
    for (int r = 0; r < R; r++) {
        const float box = s->reps[r].sim_size;
        // replica r's records, as sc_generate_scene writes them for a sim of its own
        for (int32_t g = 0; g < n_groups; g++) {
            const sc_gen_group &G = gg[(size_t)g];
            const int per = (G.kind == SC_SCENE_COMPLEXES || G.kind == SC_SCENE_WRAPPED_CHAINS) ? G.unit : 1;
            if (G.count > 0)
                k_gen_scene<<<nb_of(G.count), SC_THREADS, 0, s->st>>>(s->staging, G, per, box, seeds[r]);
        }
        if (n > 0)
            k_unpack_particles<<<nb_of(n), SC_THREADS, 0, s->st>>>(s->staging, n, n, shift_p(B.p[0], (size_t)offP[r]));
        if (nm > 0) {
            k_gen_metabolic<<<nb_of(nm), SC_THREADS, 0, s->st>>>(s->staging, nm, box, s->cfg.num_metabolites,
                                                                 mt->radius, mt->hydrophobic, seeds[r]);
            if ((rc = mc_prepare(s, nm))) return rc;
            // generated metabolic records all share one value of each untouched field
            if (r == 0) {
                uniform = B.mcUniform;
                lscs0 = B.mcLscs0;
                spoly0 = B.mcSpoly0;
            }
            if (!B.mcUniform || !uniform || B.mcLscs0 != lscs0 || B.mcSpoly0 != spoly0)
                return set_err(s, SC_E_INVALID, "generated metabolic records differ between replicas");
            k_unpack_metabolic<<<nb_of(nm), SC_THREADS, 0, s->st>>>(
                s->staging, nm, nm, s->P.SP, shift_m(B.m[0], (size_t)offM[r], Q), nullptr, nullptr, nullptr, nullptr,
                offM[r]);
        }
        // the staging buffer is rewritten by the next replica
        SC_CK(s, cudaStreamSynchronize(s->st));
        if ((rc = check_launch(s))) return rc;
    }
    // the slots past the last replica's items are empty
    if (N > offP[R])
        k_unpack_particles<<<nb_of(N - offP[R]), SC_THREADS, 0, s->st>>>(s->staging, 0, N - offP[R],
                                                                         shift_p(B.p[0], (size_t)offP[R]));
    if (Nm > offM[R])
        k_unpack_metabolic<<<nb_of(Nm - offM[R]), SC_THREADS, 0, s->st>>>(
            s->staging, 0, Nm - offM[R], s->P.SP, shift_m(B.m[0], (size_t)offM[R], Q), nullptr, nullptr, nullptr,
            nullptr, offM[R]);
    if (nm == 0) B.mcUniform = true;
    ScCounters c;
    memset(&c, 0, sizeof c);
    c.nActive = offP[R];
    c.lastActive = offP[R] - 1;
    c.nActiveM = offM[R];
    SC_CK(s, cudaMemcpyAsync(B.ctr, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    if ((rc = check_launch(s))) return rc;
    release_staging(s);
    s->loaded = true;
    return set_batch_reps(s, offP, offM);
}

int sc_mark_positions(sc_sim *s) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    enter(s);
    ScCounters c;
    SC_CK(s, cudaStreamSynchronize(s->st));
    SC_CK(s, cudaMemcpy(&c, s->B.ctr, sizeof c, cudaMemcpyDeviceToHost));
    const int capP = std::max(std::max(s->P.N, c.nextId), 1), capM = std::max(s->P.Nm, 1);
    if (capP > s->markCapP) {
        if (s->markP) {
            forget_alloc(s, (void *)s->markP);
            cudaFreeAsync(s->markP, s->st);
            s->markP = nullptr;
        }
        int rc = dalloc(s, &s->markP, (size_t)capP);
        if (rc) return rc;
        s->markCapP = capP;
    }
    if (!s->markM) {
        int rc = dalloc(s, &s->markM, (size_t)capM);
        if (rc) return rc;
        s->markCapM = capM;
    }
    ScBuffers &B = s->B;
    SC_CK(s, cudaMemsetAsync(s->markP, 0, (size_t)s->markCapP * sizeof(float4), s->st));
    SC_CK(s, cudaMemsetAsync(s->markM, 0, (size_t)s->markCapM * sizeof(float4), s->st));
    if (s->P.N > 0) sc_launch_mark(s->st, &B.ctr->nActive, B.P().pos, B.P().info, s->markP, s->markCapP);
    if (s->P.Nm > 0) sc_launch_mark(s->st, &B.ctr->nActiveM, B.M().pos, B.M().info, s->markM, s->markCapM);
    SC_CK(s, cudaStreamSynchronize(s->st));
    return check_launch(s);
}

int sc_observe(sc_sim *s, sc_observables *out) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    if (!s || !out) return set_err(s, SC_E_INVALID, "null argument");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    enter(s);
    const int cols = sc_observe_cols(), rows = sc_observe_rows();
    if (!s->obs) {
        int rc = dalloc(s, &s->obs, (size_t)(rows + 2) * cols);
        if (rc) return rc;
    }
    ScBuffers &B = s->B;
    double *res = s->obs + (size_t)rows * cols;
    SC_CK(s, cudaMemsetAsync(res, 0, 2 * (size_t)cols * sizeof(double), s->st));
    const double box = s->cfg.sim_size;
    if (s->P.N > 0) {
        PFields F = B.P();
        sc_launch_observe(s->st, &B.ctr->nActive, F.pos, F.vel, F.info, F.nb, nullptr, 0, 0, s->markP, s->markCapP,
                          box, s->P.periodic, s->obs, res);
    }
    if (s->P.Nm > 0) {
        MFields M = B.M();
        sc_launch_observe(s->st, &B.ctr->nActiveM, M.pos, M.vel, M.info, nullptr,
                          reinterpret_cast<const float *>(M.met), s->P.SP, s->P.S, s->markM, s->markCapM, box,
                          s->P.periodic, s->obs, res + cols);
    }
    std::vector<double> h((size_t)2 * cols);
    SC_CK(s, cudaMemcpyAsync(h.data(), res, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    memset(out, 0, sizeof *out);
    for (int k = 0; k < 2; k++) {
        const double *r = &h[(size_t)k * cols];
        out->msd_items[k] = (int64_t)r[1];
        out->msd[k] = r[1] > 0 ? r[0] / r[1] : 0.0;
        out->active[k] = (int64_t)r[3];
        out->mean_v2[k] = r[3] > 0 ? r[2] / r[3] : 0.0;
    }
    out->bond_slots = (int64_t)h[4];
    for (int m = 0; m < SC_AOS_NUM_METABOLITES; m++) out->metabolites[m] = h[(size_t)cols + 5 + m];
    return check_launch(s);
}

int sc_pair_histogram(sc_sim *s, int32_t type_a, int32_t type_b, float r_max, int32_t n_bins, uint64_t *counts) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    if (!s || !counts) return set_err(s, SC_E_INVALID, "null argument");
    if (!s->loaded) return set_err(s, SC_E_STATE, "no state loaded");
    if (n_bins < 1 || n_bins > 4096) return set_err(s, SC_E_INVALID, "n_bins must be in 1..4096");
    if (!(r_max > 0.0f) || r_max > s->cfg.grid_cell_size)
        return set_err(s, SC_E_INVALID, "r_max must be in (0, grid cell size]");
    enter(s);
    int rc;
    if (!(s->P.binned & SC_BINNED_P) && (rc = run_phase(s, SC_PHASE_SORT_PARTICLES, 0))) return rc;
    ScBuffers &B = s->B;
    unsigned long long *d = nullptr;
    SC_CK(s, cudaMallocAsync((void **)&d, (size_t)n_bins * sizeof(unsigned long long), s->st));
    SC_CK(s, cudaMemsetAsync(d, 0, (size_t)n_bins * sizeof(unsigned long long), s->st));
    if (s->P.N > 0) {
        PFields F = B.P();
        sc_launch_pair_histogram(s->st, s->P, B.cellStartP, &B.ctr->nActive, F.pos, F.info, type_a, type_b,
                                 (double)r_max, n_bins, d, s->gridCap);
    }
    SC_CK(s, cudaMemcpyAsync(counts, d, (size_t)n_bins * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->st));
    SC_CK(s, cudaFreeAsync(d, s->st));
    SC_CK(s, cudaStreamSynchronize(s->st));
    return check_launch(s);
}

int sc_checkpoint_write(sc_sim *s, void *file) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    if (!s || !file) return set_err(s, SC_E_INVALID, "null argument");
    sc_counters c;
    int rc = sc_get_counters(s, &c);
    if (rc) return rc;
    std::vector<sc_particle> p((size_t)std::max(s->P.N, 1));
    std::vector<sc_metabolic_particle> m((size_t)std::max(s->P.Nm, 1));
    if ((rc = sc_export_state(s, p.data(), m.data()))) return rc;
    FILE *f = (FILE *)file;
    const int32_t hdr[6] = {0, 0, c.n_active_particles, c.n_active_metabolic_particles, c.step, c.next_particle_id};
    char magic[8] = {'S', 'C', 'C', 'K', 'P', 'T', '0', '1'};
    if (fwrite(magic, 1, 8, f) != 8 || fwrite(hdr + 2, sizeof(int32_t), 4, f) != 4 ||
        fwrite(p.data(), sizeof(sc_particle), (size_t)c.n_active_particles, f) != (size_t)c.n_active_particles ||
        fwrite(m.data(), sizeof(sc_metabolic_particle), (size_t)c.n_active_metabolic_particles, f) !=
            (size_t)c.n_active_metabolic_particles)
        return set_err(s, SC_E_IO, "checkpoint write failed");
    return SC_OK;
}

int sc_checkpoint_read(sc_sim *s, void *file) {
    if (s && !s->reps.empty()) return set_err(s, SC_E_INVALID, "not available on a batched sim");
    if (!s || !file) return set_err(s, SC_E_INVALID, "null argument");
    FILE *f = (FILE *)file;
    char magic[8];
    int32_t hdr[4];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "SCCKPT01", 8) != 0 || fread(hdr, sizeof(int32_t), 4, f) != 4)
        return set_err(s, SC_E_IO, "not a checkpoint");
    const int32_t n = hdr[0], nm = hdr[1];
    if (n < 0 || nm < 0 || n > s->P.N || nm > s->P.Nm)
        return set_err(s, SC_E_INVALID, "checkpoint holds more items than the sim's capacity");
    std::vector<sc_particle> p((size_t)std::max(n, 1));
    std::vector<sc_metabolic_particle> m((size_t)std::max(nm, 1));
    if (fread(p.data(), sizeof(sc_particle), (size_t)n, f) != (size_t)n ||
        fread(m.data(), sizeof(sc_metabolic_particle), (size_t)nm, f) != (size_t)nm)
        return set_err(s, SC_E_IO, "truncated checkpoint");
    return sc_load_state(s, p.data(), n, m.data(), nm, hdr[2], hdr[3]);
}

int64_t sc_reduce_frame_async(sc_sim *s, sc_reduced_particle *particles, sc_reduced_metabolic_particle *metabolic) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    enter(s);
    const int slot = (int)(s->frames & 1);
    int rc = ensure_frame_slots(s);
    if (rc) return rc;
    // the slot's previous frame must have left the device before it is rewritten
    if (s->frames >= 2) SC_CK(s, cudaStreamWaitEvent(s->st, s->copied[slot], 0));
    ScLaunchCtx c = ctx(s);
    sc_phase_reduce(c, slot);
    rc = check_launch(s);
    if (rc) return rc;
    SC_CK(s, cudaEventRecord(s->reduced[slot], s->st));
    SC_CK(s, cudaStreamWaitEvent(s->copySt, s->reduced[slot], 0));
    if (particles && s->P.N > 0)
        SC_CK(s, cudaMemcpyAsync(particles, slot ? s->B.redP2 : s->B.redP,
                                 (size_t)s->P.N * sizeof(sc_reduced_particle), cudaMemcpyDeviceToHost, s->copySt));
    if (metabolic && s->P.Nm > 0)
        SC_CK(s, cudaMemcpyAsync(metabolic, slot ? s->B.redM2 : s->B.redM,
                                 (size_t)s->P.Nm * sizeof(sc_reduced_metabolic_particle), cudaMemcpyDeviceToHost,
                                 s->copySt));
    SC_CK(s, cudaEventRecord(s->copied[slot], s->copySt));
    return s->frames++;
}

int sc_frame_wait(sc_sim *s, int64_t ticket) {
    if (!s) return set_err(nullptr, SC_E_INVALID, "null sim");
    if (ticket < 0 || ticket >= s->frames) return set_err(s, SC_E_INVALID, "no such frame");
    enter(s);
    // The slot's event records this frame's copy or a later one on the same
    // in-order copy stream; either way this frame has landed when it fires.
    SC_CK(s, cudaEventSynchronize(s->copied[ticket & 1]));
    return check_launch(s);
}

}  // extern "C"
