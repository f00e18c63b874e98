// ref_device.cu -- TEST INFRASTRUCTURE ONLY (oracle).
//
// Runs the reference's own CUDA step on the GPU: loads the reference's
// kernels from oracle/_ref/ref_step.cubin (oracle/ref_device_kernels.cu,
// built where the reference tree is present) and replays the launch
// sequence of spatial_cell_sim/src/main.cu:284-661 around them as main()
// does, on the legacy default stream:
//   * the reference's buffers: double-buffered 256 / 304-byte structs, key
//     and cell-range arrays, one curandState per slot (memory.cuh,
//     main.cu:225-243);
//   * updateGridAndSort (grid.cuh:111-139): updateIndices, a device
//     synchronisation, the CUDA toolkit's cub::DeviceRadixSort::SortPairs of
//     (key, whole struct) over all 32 key bits and the whole capacity, a
//     memset of the cell ranges, updateGridRanges;
//   * a memset of the next buffer before every double-buffered kernel
//     (clearNextOnDevice), the cudaDeviceSynchronize calls and the
//     nActiveParticles read-backs of main.cu:367-371, 397-399, 615-616, and
//     launch sizes of CUDA_NUM_BLOCKS(count) x 256 from the host copies;
//   * frame persistence is not run (the step is timed without it).
// Philox-compatible noise: before each Brownian kernel a harness kernel
// writes every slot's counter position {seed, id of the item in the slot,
// step} (the reference seeds XORWOW per slot once, main.cu:54-66).
//
// The reference indexes outside its buffers in a few places (documented
// with the CPU oracle): updateGridRanges stores to gridRanges[-2..-1] where
// the active items end (grid.cuh:61-72), and polymerize can store to
// particles[-1] / interactions[-1] at a chain end.  Every buffer here is
// allocated with guard elements before and after it, so those stores land
// in memory the harness owns; refdev_guards reports which guards were
// written.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "spatialcell.h"

namespace {

struct alignas(16) Blob256 { uint4 w[16]; };
struct alignas(16) Blob304 { uint4 w[19]; };
static_assert(sizeof(Blob256) == sizeof(sc_particle) && sizeof(Blob304) == sizeof(sc_metabolic_particle), "layouts");

// config.cuh:15-44 (the reference's Config, copied to __constant__ d_Config)
struct RefConfig {
    int numParticles, numMetabolicParticles, steps;
    float simSize, maxInteractionDistance, maxDiffusionDistance, gridCellSize;
    int nGridCells, nGridCellsBits;
    float totalGridCells;
    float movementNoiseScale, rotationNoiseScale, metaboliteMovementNoiseScale, velocityDecay, angularVelocityDecay;
    int noiseCoordinationSteps, relaxationSteps, metaboliteDiffusionSteps, persistEveryNthFrame, reportEveryNthFrame;
};

const int kThreads = 256;             // CUDA_THREADS_PER_BLOCK, constants.cuh:34
const size_t kGuardBytes = 4096;      // guard before and after every buffer
const int kRngBytes = 32;             // the harness curandState (shim_dev/curand_kernel.h)
const uint32_t kStreamPU = 0, kStreamPN = 1, kStreamMU = 2, kStreamMN = 3;  // scmath.h SC_STREAM_*

thread_local std::string g_err;

}  // namespace

struct refdev_sim {
    CUmodule mod = nullptr;
    std::map<std::string, CUfunction> fn;
    RefConfig cfg;
    int N = 0, Nm = 0;
    uint64_t seed = 0;
    size_t cells = 0;
    std::vector<void *> bases;  // allocation bases (guard in front)
    struct Guarded { char *base; size_t bytes; };
    std::map<std::string, Guarded> guards;
    char *pCur = nullptr, *pNext = nullptr, *mCur = nullptr, *mNext = nullptr;
    unsigned *keysP = nullptr, *keysP2 = nullptr, *keysM = nullptr, *keysM2 = nullptr;
    unsigned *rangesP = nullptr, *rangesM = nullptr;
    char *rngP = nullptr, *rngM = nullptr;
    char *types = nullptr, *flat = nullptr, *prules = nullptr;
    int *pidx = nullptr;
    int *dNActive = nullptr, *dLastActive = nullptr, *dNextId = nullptr, *dCount = nullptr;
    void *sortTempP = nullptr, *sortTempM = nullptr;
    size_t sortBytesP = 0, sortBytesM = 0;
    char *redP = nullptr, *redM = nullptr;
    int hActive = 0, hActiveM = 0, step = 0;
    std::string err;
};

namespace {

int fail(refdev_sim *s, const std::string &m) {
    if (s) s->err = m;
    g_err = m;
    return -1;
}

#define RD_CK(s, call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return fail((s), std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define RD_CU(s, call)                                                                         \
    do {                                                                                       \
        CUresult r_ = (call);                                                                  \
        if (r_ != CUDA_SUCCESS) {                                                              \
            const char *m_ = nullptr;                                                          \
            cuGetErrorString(r_, &m_);                                                         \
            return fail((s), std::string(#call) + ": " + (m_ ? m_ : "?"));                     \
        }                                                                                      \
    } while (0)

// bytes of device memory with kGuardBytes of zeroed guard on both sides
int galloc(refdev_sim *s, const char *name, size_t bytes, void **out) {
    char *base = nullptr;
    const size_t total = bytes + 2 * kGuardBytes;
    RD_CK(s, cudaMalloc((void **)&base, total));
    RD_CK(s, cudaMemset(base, 0, total));
    s->bases.push_back(base);
    s->guards[name] = {base, bytes};
    *out = base + kGuardBytes;
    return 0;
}

int launch(refdev_sim *s, const char *name, long long nthreads, std::vector<void *> args) {
    if (nthreads <= 0) return 0;  // a launch of zero blocks does nothing
    auto it = s->fn.find(name);
    if (it == s->fn.end()) return fail(s, std::string("no kernel ") + name);
    const unsigned blocks = (unsigned)((nthreads + kThreads - 1) / kThreads);  // CUDA_NUM_BLOCKS
    RD_CU(s, cuLaunchKernel(it->second, blocks, 1, 1, kThreads, 1, 1, 0, nullptr, args.data(), nullptr));
    return 0;
}

int sync(refdev_sim *s) {
    RD_CK(s, cudaDeviceSynchronize());
    return 0;
}

int read_active(refdev_sim *s) {  // nActiveParticles.copyToHost()
    RD_CK(s, cudaMemcpy(&s->hActive, s->dNActive, sizeof(int), cudaMemcpyDeviceToHost));
    return 0;
}

int set_rng(refdev_sim *s, bool metabolic) {
    char *st = metabolic ? s->rngM : s->rngP;
    char *items = metabolic ? s->mCur : s->pCur;
    int stride = metabolic ? (int)sizeof(sc_metabolic_particle) : (int)sizeof(sc_particle);
    int n = metabolic ? s->Nm : s->N;
    unsigned long long seed = s->seed;
    int step = s->step;
    unsigned su = metabolic ? kStreamMU : kStreamPU, sn = metabolic ? kStreamMN : kStreamPN;
    return launch(s, "ref_set_rng", n, {&st, &items, &stride, &n, &seed, &step, &su, &sn});
}

// updateGridAndSort (grid.cuh:111-139)
template <class Blob>
int sort_set(refdev_sim *s, char *&cur, char *&next, unsigned *&keys, unsigned *&keys2, unsigned *ranges, int n,
             void *temp, size_t tempBytes, const char *keyKernel) {
    if (launch(s, keyKernel, n, {&cur, &keys, &n})) return -1;
    if (sync(s)) return -1;
    size_t bytes = tempBytes;
    RD_CK(s, cub::DeviceRadixSort::SortPairs(temp, bytes, keys, keys2, (const Blob *)cur, (Blob *)next, n));
    std::swap(cur, next);
    std::swap(keys, keys2);
    RD_CK(s, cudaMemset(ranges, 0, s->cells * 2 * sizeof(unsigned)));
    long long total = (long long)s->cfg.totalGridCells;
    return launch(s, "ref_updateGridRanges", total, {&keys, &ranges, &n});
}

int clear_next(refdev_sim *s, bool metabolic) {  // clearNextOnDevice()
    if (metabolic) RD_CK(s, cudaMemset(s->mNext, 0, (size_t)s->Nm * sizeof(sc_metabolic_particle)));
    else RD_CK(s, cudaMemset(s->pNext, 0, (size_t)s->N * sizeof(sc_particle)));
    return 0;
}

}  // namespace

extern "C" {

const char *refdev_last_error(const refdev_sim *s) { return s ? s->err.c_str() : g_err.c_str(); }

void refdev_destroy(refdev_sim *s) {
    if (!s) return;
    cudaDeviceSynchronize();
    for (void *b : s->bases) cudaFree(b);
    if (s->sortTempP) cudaFree(s->sortTempP);
    if (s->sortTempM) cudaFree(s->sortTempM);
    if (s->mod) cuModuleUnload(s->mod);
    delete s;
}

refdev_sim *refdev_create(const char *cubin, const sc_config *c, const sc_type_info *types, int n_types,
                          const sc_rule *rules, int n_rules) {
    refdev_sim *s = new refdev_sim();
    auto bail = [&](const std::string &m) {
        g_err = m + (s->err.empty() ? "" : ": " + s->err);
        refdev_destroy(s);
        return (refdev_sim *)nullptr;
    };
    if (cudaFree(nullptr) != cudaSuccess) return bail("no CUDA context");  // the runtime's primary context
    if (cuModuleLoad(&s->mod, cubin) != CUDA_SUCCESS) return bail(std::string("cannot load ") + cubin);
    const char *names[] = {"ref_updateIndices_P", "ref_updateIndices_M", "ref_updateGridRanges", "ref_move",
                           "ref_brownian_P", "ref_brownian_M", "ref_moveMetabolicParticles", "ref_coordinateNoise",
                           "ref_applyNoise_P", "ref_applyNoise_M", "ref_relax", "ref_relaxMetabolicParticles",
                           "ref_relaxMetabolicParticlePartners", "ref_applyVelocities_P", "ref_applyVelocities_M",
                           "ref_complexify", "ref_transitionInteractions", "ref_polymerize", "ref_diffuseMetabolites",
                           "ref_removeInterferingMetabolicParticles", "ref_reduce_P", "ref_reduce_M", "ref_set_rng",
                           "ref_count_nonfinite"};
    for (const char *nm : names) {
        CUfunction f;
        if (cuModuleGetFunction(&f, s->mod, nm) != CUDA_SUCCESS) return bail(std::string("kernel missing: ") + nm);
        s->fn[nm] = f;
    }
    // layouts of the cubin's structs against this side's view of them
    {
        CUdeviceptr p;
        size_t bytes;
        int lay[8];
        if (cuModuleGetGlobal(&p, &bytes, s->mod, "ref_layout") != CUDA_SUCCESS || bytes != sizeof lay ||
            cuMemcpyDtoH(lay, p, sizeof lay) != CUDA_SUCCESS)
            return bail("layout table missing");
        const int want[8] = {(int)sizeof(sc_particle), (int)sizeof(sc_metabolic_particle),
                             (int)sizeof(sc_reduced_particle), (int)sizeof(sc_reduced_metabolic_particle),
                             (int)sizeof(sc_rule), (int)sizeof(sc_type_info), (int)sizeof(RefConfig), kRngBytes};
        if (memcmp(lay, want, sizeof lay) != 0) return bail("struct layouts of the cubin differ");
    }
    // Config(Json::Value), config.cuh:46-75
    RefConfig &k = s->cfg;
    memset(&k, 0, sizeof k);
    k.numParticles = c->num_particles;
    k.numMetabolicParticles = c->num_metabolic_particles;
    k.steps = c->steps;
    k.simSize = c->sim_size;
    k.maxInteractionDistance = c->max_interaction_distance;
    k.maxDiffusionDistance = c->max_diffusion_distance;
    k.gridCellSize = c->grid_cell_size;
    k.nGridCells = (int)ceilf(k.simSize / k.gridCellSize);
    k.nGridCellsBits = 1;
    int p2 = 2;
    while (p2 < k.nGridCells) { p2 *= 2; k.nGridCellsBits++; }
    k.nGridCells = p2;
    k.totalGridCells = (float)(k.nGridCells * k.nGridCells * k.nGridCells);
    k.movementNoiseScale = c->movement_noise_scale;
    k.rotationNoiseScale = c->rotation_noise_scale;
    k.metaboliteMovementNoiseScale = c->metabolite_movement_noise_scale;
    k.velocityDecay = c->velocity_decay;
    k.angularVelocityDecay = c->angular_velocity_decay;
    k.noiseCoordinationSteps = c->noise_coordination_steps;
    k.relaxationSteps = c->relaxation_steps;
    k.metaboliteDiffusionSteps = c->metabolite_diffusion_steps;
    k.persistEveryNthFrame = c->persist_every_nth_frame;
    k.reportEveryNthFrame = c->report_every_nth_frame;
    {
        CUdeviceptr p;
        size_t bytes;
        if (cuModuleGetGlobal(&p, &bytes, s->mod, "d_Config") != CUDA_SUCCESS || bytes != sizeof k ||
            cuMemcpyHtoD(p, &k, sizeof k) != CUDA_SUCCESS)  // cudaMemcpyToSymbol(d_Config), main.cu:256
            return bail("d_Config");
    }
    s->N = c->num_particles;
    s->Nm = c->num_metabolic_particles;
    s->seed = c->seed;
    s->cells = (size_t)k.nGridCells * k.nGridCells * k.nGridCells;
    const size_t N = (size_t)std::max(s->N, 1), Nm = (size_t)std::max(s->Nm, 1);
    void *v;
#define GA(name, bytes, dst, T) \
    if (galloc(s, name, bytes, &v)) return bail("allocation"); \
    dst = (T)v;
    GA("particles0", N * sizeof(sc_particle), s->pCur, char *);
    GA("particles1", N * sizeof(sc_particle), s->pNext, char *);
    GA("metabolic0", Nm * sizeof(sc_metabolic_particle), s->mCur, char *);
    GA("metabolic1", Nm * sizeof(sc_metabolic_particle), s->mNext, char *);
    GA("keysP0", N * 4, s->keysP, unsigned *);
    GA("keysP1", N * 4, s->keysP2, unsigned *);
    GA("keysM0", Nm * 4, s->keysM, unsigned *);
    GA("keysM1", Nm * 4, s->keysM2, unsigned *);
    GA("rangesP", s->cells * 8, s->rangesP, unsigned *);
    GA("rangesM", s->cells * 8, s->rangesM, unsigned *);
    GA("rngP", N * kRngBytes, s->rngP, char *);
    GA("rngM", Nm * kRngBytes, s->rngM, char *);
    GA("counters", 4 * sizeof(int), s->dNActive, int *);
    s->dLastActive = s->dNActive + 1;
    s->dNextId = s->dNActive + 2;
    s->dCount = s->dNActive + 3;
    GA("reducedP", N * sizeof(sc_reduced_particle), s->redP, char *);
    GA("reducedM", Nm * sizeof(sc_reduced_metabolic_particle), s->redM, char *);
    // tables: id-indexed types; id-indexed rules (the first of duplicate ids);
    // the partner index, 2 * (max rule id + 1) ints, with the rules of a type
    // in ascending id order (interactions.cuh:59-145)
    std::vector<sc_type_info> ty((size_t)std::max(n_types, 1));
    if (n_types > 0) memcpy(ty.data(), types, (size_t)n_types * sizeof(sc_type_info));
    int maxId = 0;
    for (int i = 0; i < n_rules; i++) maxId = std::max(maxId, rules[i].id);
    std::vector<sc_rule> flat((size_t)maxId + 1);
    memset(flat.data(), 0, flat.size() * sizeof(sc_rule));
    std::vector<char> seen((size_t)maxId + 1, 0);
    for (int i = 0; i < n_rules; i++) {
        if (rules[i].id < 0 || seen[(size_t)rules[i].id]) continue;
        seen[(size_t)rules[i].id] = 1;
        flat[(size_t)rules[i].id] = rules[i];
    }
    std::map<int, std::vector<int>> byType;
    for (int id = 0; id <= maxId; id++) {
        if (!seen[(size_t)id]) continue;
        if (flat[(size_t)id].first_partner_type >= 0) byType[flat[(size_t)id].first_partner_type].push_back(id);
        if (flat[(size_t)id].second_partner_type >= 0) byType[flat[(size_t)id].second_partner_type].push_back(id);
    }
    std::vector<int> pidx(((size_t)maxId + 1) * 2, 0);
    std::vector<sc_rule> pr;
    for (auto &kv : byType) {
        int start = (int)pr.size();
        for (int id : kv.second) pr.push_back(flat[(size_t)id]);
        if ((size_t)kv.first * 2 + 1 < pidx.size()) {
            pidx[(size_t)kv.first * 2] = start;
            pidx[(size_t)kv.first * 2 + 1] = (int)pr.size();
        }
    }
    if (pr.empty()) pr.resize(1);
    GA("types", ty.size() * sizeof(sc_type_info), s->types, char *);
    GA("flatRules", flat.size() * sizeof(sc_rule), s->flat, char *);
    GA("partnerIndex", pidx.size() * sizeof(int), s->pidx, int *);
    GA("partnerRules", pr.size() * sizeof(sc_rule), s->prules, char *);
#undef GA
    if (cudaMemcpy(s->types, ty.data(), ty.size() * sizeof(sc_type_info), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->flat, flat.data(), flat.size() * sizeof(sc_rule), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->pidx, pidx.data(), pidx.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->prules, pr.data(), pr.size() * sizeof(sc_rule), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail("table upload");
    // RadixSortPairs: temporary storage sized once for the capacity (grid.cuh:76-96)
    if (cub::DeviceRadixSort::SortPairs(nullptr, s->sortBytesP, s->keysP, s->keysP2, (const Blob256 *)s->pCur,
                                        (Blob256 *)s->pNext, s->N) != cudaSuccess ||
        cub::DeviceRadixSort::SortPairs(nullptr, s->sortBytesM, s->keysM, s->keysM2, (const Blob304 *)s->mCur,
                                        (Blob304 *)s->mNext, s->Nm) != cudaSuccess)
        return bail("SortPairs sizing");
    if (cudaMalloc(&s->sortTempP, std::max<size_t>(s->sortBytesP, 1)) != cudaSuccess ||
        cudaMalloc(&s->sortTempM, std::max<size_t>(s->sortBytesM, 1)) != cudaSuccess)
        return bail("SortPairs storage");
    if (cudaDeviceSynchronize() != cudaSuccess) return bail("create");
    return s;
}

int refdev_load_state(refdev_sim *s, const sc_particle *p, int n, const sc_metabolic_particle *m, int nm, int step,
                      int next_id) {
    if (n > s->N || nm > s->Nm || n < 0 || nm < 0) return fail(s, "state larger than the capacity");
    RD_CK(s, cudaMemset(s->pCur, 0, (size_t)s->N * sizeof(sc_particle)));
    RD_CK(s, cudaMemset(s->mCur, 0, (size_t)s->Nm * sizeof(sc_metabolic_particle)));
    if (n) RD_CK(s, cudaMemcpy(s->pCur, p, (size_t)n * sizeof(sc_particle), cudaMemcpyHostToDevice));
    if (nm) RD_CK(s, cudaMemcpy(s->mCur, m, (size_t)nm * sizeof(sc_metabolic_particle), cudaMemcpyHostToDevice));
    int ctr[4] = {n, n - 1, next_id, 0};
    RD_CK(s, cudaMemcpy(s->dNActive, ctr, sizeof ctr, cudaMemcpyHostToDevice));
    s->hActive = n;
    s->hActiveM = nm;
    s->step = step;
    return sync(s);
}

// One kernel (or kernel pair) of main.cu's loop, as main() launches it.
int refdev_run_phase(refdev_sim *s, int phase, int arg) {
    int step = s->step;
    int n = s->hActive, nm = s->hActiveM;
    int *na = s->dNActive, *la = s->dLastActive, *ni = s->dNextId;
    switch (phase) {
        case SC_PHASE_SORT_PARTICLES:  // grid.cuh:111-139, then main.cu:367-371
            if (sort_set<Blob256>(s, s->pCur, s->pNext, s->keysP, s->keysP2, s->rangesP, s->N, s->sortTempP,
                                  s->sortBytesP, "ref_updateIndices_P") || sync(s) || read_active(s))
                return -1;
            {
                int last = s->hActive - 1;
                RD_CK(s, cudaMemcpy(s->dLastActive, &last, sizeof(int), cudaMemcpyHostToDevice));
            }
            return 0;
        case SC_PHASE_SORT_METABOLIC:
            if (sort_set<Blob304>(s, s->mCur, s->mNext, s->keysM, s->keysM2, s->rangesM, s->Nm, s->sortTempM,
                                  s->sortBytesM, "ref_updateIndices_M"))
                return -1;
            return sync(s);
        case SC_PHASE_MOVE_BROWNIAN: {  // main.cu:374-399
            if (clear_next(s, false)) return -1;
            if (launch(s, "ref_move", n, {&step, &s->rngP, &s->pCur, &s->pNext, &n, &na, &la, &ni, &s->rangesP}))
                return -1;
            std::swap(s->pCur, s->pNext);
            float scale = s->cfg.movementNoiseScale;
            if (set_rng(s, false) || launch(s, "ref_brownian_P", n, {&step, &s->rngP, &s->pCur, &n, &scale}))
                return -1;
            return sync(s) || read_active(s);
        }
        case SC_PHASE_MOVE_BROWNIAN_METAB: {  // main.cu:401-420
            if (clear_next(s, true)) return -1;
            if (launch(s, "ref_moveMetabolicParticles", nm, {&step, &s->rngM, &s->mCur, &s->mNext, &nm, &s->rangesM}))
                return -1;
            std::swap(s->mCur, s->mNext);
            float scale = s->cfg.metaboliteMovementNoiseScale;
            if (set_rng(s, true) || launch(s, "ref_brownian_M", nm, {&step, &s->rngM, &s->mCur, &nm, &scale}))
                return -1;
            return sync(s);
        }
        case SC_PHASE_COORDINATE_NOISE: {  // main.cu:425-440
            if (clear_next(s, false)) return -1;
            float frac = (float)arg / s->cfg.noiseCoordinationSteps;
            if (launch(s, "ref_coordinateNoise", n, {&step, &s->rngP, &s->pCur, &s->pNext, &n, &s->rangesP, &frac}))
                return -1;
            std::swap(s->pCur, s->pNext);
            return sync(s);
        }
        case SC_PHASE_APPLY_NOISE:  // main.cu:442-454
            if (launch(s, "ref_applyNoise_P", n, {&step, &s->rngP, &s->pCur, &n}) ||
                launch(s, "ref_applyNoise_M", nm, {&step, &s->rngM, &s->mCur, &nm}))
                return -1;
            return sync(s);
        case SC_PHASE_RELAX:  // main.cu:478-496
            if (clear_next(s, false) ||
                launch(s, "ref_relax", n, {&step, &s->rngP, &s->pCur, &s->pNext, &n, &s->rangesP, &s->flat}))
                return -1;
            std::swap(s->pCur, s->pNext);
            return sync(s);
        case SC_PHASE_RELAX_METAB:  // main.cu:508-521
            if (clear_next(s, true) ||
                launch(s, "ref_relaxMetabolicParticles", nm,
                       {&step, &s->rngM, &s->mCur, &s->mNext, &nm, &s->rangesM, &s->pCur, &s->rangesP}))
                return -1;
            std::swap(s->mCur, s->mNext);
            return 0;
        case SC_PHASE_RELAX_PARTNERS:  // main.cu:524-537, then the synchronisation of main.cu:540
            if (clear_next(s, false) ||
                launch(s, "ref_relaxMetabolicParticlePartners", n,
                       {&step, &s->rngP, &s->pCur, &s->pNext, &n, &s->rangesP, &s->mCur, &s->rangesM}))
                return -1;
            std::swap(s->pCur, s->pNext);
            return sync(s);
        case SC_PHASE_APPLY_VELOCITIES: {  // main.cu:548-562
            float f = 0.45f;
            if (launch(s, "ref_applyVelocities_P", n, {&step, &s->rngP, &s->pCur, &n, &f}) ||
                launch(s, "ref_applyVelocities_M", nm, {&step, &s->rngM, &s->mCur, &nm, &f}))
                return -1;
            return sync(s);
        }
        case SC_PHASE_COMPLEXIFY: {  // main.cu:567-579 (step argument -1 at start-up, main.cu:325)
            int st = arg == -1 ? -1 : step;
            if (clear_next(s, false) ||
                launch(s, "ref_complexify", n,
                       {&st, &s->rngP, &s->pCur, &s->pNext, &n, &s->rangesP, &s->flat, &s->pidx, &s->prules}))
                return -1;
            std::swap(s->pCur, s->pNext);
            return 0;
        }
        case SC_PHASE_TRANSITION:  // main.cu:582-598
            if (clear_next(s, false) ||
                launch(s, "ref_transitionInteractions", n,
                       {&step, &s->rngP, &s->pCur, &s->pNext, &n, &na, &la, &ni, &s->rangesP, &s->types, &s->flat,
                        &s->pidx, &s->prules}))
                return -1;
            std::swap(s->pCur, s->pNext);
            return 0;
        case SC_PHASE_POLYMERIZE:  // main.cu:600-616
            if (launch(s, "ref_polymerize", n,
                       {&step, &s->rngP, &s->pCur, &n, &na, &la, &ni, &s->rangesP, &s->types, &s->flat, &s->pidx,
                        &s->prules}))
                return -1;
            return sync(s) || read_active(s) || sync(s);
        case SC_PHASE_DIFFUSE:  // main.cu:637-648
            if (clear_next(s, true) ||
                launch(s, "ref_diffuseMetabolites", nm, {&step, &s->rngM, &s->mCur, &s->mNext, &nm, &s->rangesM}))
                return -1;
            std::swap(s->mCur, s->mNext);
            return sync(s);
        case SC_PHASE_REMOVE_INTERFERING:  // main.cu:301-312
            if (clear_next(s, true) ||
                launch(s, "ref_removeInterferingMetabolicParticles", nm,
                       {&s->mCur, &s->mNext, &nm, &s->rangesM, &s->pCur, &s->rangesP}))
                return -1;
            std::swap(s->mCur, s->mNext);
            return sync(s);
        case SC_PHASE_END_STEP:
            s->step++;
            return 0;
        default:
            return fail(s, "unknown phase");
    }
}

// main.cu:284-338 (the first frame is not written)
int refdev_prepare(refdev_sim *s) {
    if (refdev_run_phase(s, SC_PHASE_SORT_PARTICLES, 0) || refdev_run_phase(s, SC_PHASE_SORT_METABOLIC, 0) ||
        refdev_run_phase(s, SC_PHASE_REMOVE_INTERFERING, 0) || refdev_run_phase(s, SC_PHASE_COMPLEXIFY, -1))
        return -1;
    return sync(s);
}

// n_steps iterations of main.cu:347-661, ending with the device synchronised.
int refdev_step(refdev_sim *s, int n_steps) {
    const RefConfig &c = s->cfg;
    for (int k = 0; k < n_steps; k++) {
        int rc = refdev_run_phase(s, SC_PHASE_SORT_PARTICLES, 0) || refdev_run_phase(s, SC_PHASE_SORT_METABOLIC, 0) ||
                 refdev_run_phase(s, SC_PHASE_MOVE_BROWNIAN, 0) || refdev_run_phase(s, SC_PHASE_MOVE_BROWNIAN_METAB, 0);
        for (int j = 0; j < c.noiseCoordinationSteps && !rc; j++) rc = refdev_run_phase(s, SC_PHASE_COORDINATE_NOISE, j);
        if (!rc) rc = refdev_run_phase(s, SC_PHASE_APPLY_NOISE, 0);
        for (int j = 0; j < c.relaxationSteps && !rc; j++) {
            rc = refdev_run_phase(s, SC_PHASE_RELAX, j);
            if (!rc && j % 2 == 0)
                rc = refdev_run_phase(s, SC_PHASE_RELAX_METAB, j) || refdev_run_phase(s, SC_PHASE_RELAX_PARTNERS, j);
        }
        if (!rc)
            rc = refdev_run_phase(s, SC_PHASE_APPLY_VELOCITIES, 0) || refdev_run_phase(s, SC_PHASE_COMPLEXIFY, 0) ||
                 refdev_run_phase(s, SC_PHASE_TRANSITION, 0) || refdev_run_phase(s, SC_PHASE_POLYMERIZE, 0);
        for (int j = 0; j < c.metaboliteDiffusionSteps && !rc; j++) rc = refdev_run_phase(s, SC_PHASE_DIFFUSE, j);
        if (!rc) rc = refdev_run_phase(s, SC_PHASE_END_STEP, 0);
        if (rc) return -1;
    }
    return sync(s);
}

int refdev_export_state(refdev_sim *s, sc_particle *p, sc_metabolic_particle *m) {
    if (p && s->N) RD_CK(s, cudaMemcpy(p, s->pCur, (size_t)s->N * sizeof(sc_particle), cudaMemcpyDeviceToHost));
    if (m && s->Nm)
        RD_CK(s, cudaMemcpy(m, s->mCur, (size_t)s->Nm * sizeof(sc_metabolic_particle), cudaMemcpyDeviceToHost));
    return 0;
}

// The cell ranges of the last sort (gridRanges layout); the reference keeps
// no permutation, so perm is filled with 0xFFFFFFFF.
int refdev_export_grid(refdev_sim *s, int which, uint32_t *ranges, uint32_t *perm) {
    if (ranges) RD_CK(s, cudaMemcpy(ranges, which ? s->rangesM : s->rangesP, s->cells * 8, cudaMemcpyDeviceToHost));
    if (perm) memset(perm, 0xff, (size_t)(which ? s->Nm : s->N) * 4);
    return 0;
}

int refdev_get_counters(refdev_sim *s, sc_counters *c) {
    int ctr[4];
    RD_CK(s, cudaMemcpy(ctr, s->dNActive, sizeof ctr, cudaMemcpyDeviceToHost));
    memset(c, 0, sizeof *c);
    c->n_active_particles = ctr[0];
    c->n_active_metabolic_particles = s->hActiveM;
    c->next_particle_id = ctr[2];
    c->step = s->step;
    return 0;
}

// main.cu:95-126: clearOnDevice + reduceParticles over the host active counts
int refdev_reduce_frame(refdev_sim *s, sc_reduced_particle *rp, sc_reduced_metabolic_particle *rm) {
    int n = s->hActive, nm = s->hActiveM;
    RD_CK(s, cudaMemset(s->redP, 0, (size_t)s->N * sizeof(sc_reduced_particle)));
    RD_CK(s, cudaMemset(s->redM, 0, (size_t)s->Nm * sizeof(sc_reduced_metabolic_particle)));
    if (launch(s, "ref_reduce_P", n, {&s->pCur, &s->redP, &n}) ||
        launch(s, "ref_reduce_M", nm, {&s->mCur, &s->redM, &nm}) || sync(s))
        return -1;
    if (rp) RD_CK(s, cudaMemcpy(rp, s->redP, (size_t)s->N * sizeof(sc_reduced_particle), cudaMemcpyDeviceToHost));
    if (rm)
        RD_CK(s, cudaMemcpy(rm, s->redM, (size_t)s->Nm * sizeof(sc_reduced_metabolic_particle), cudaMemcpyDeviceToHost));
    return 0;
}

// Active items with a non-finite position, particles and metabolic items.
int refdev_nonfinite(refdev_sim *s, int64_t out[2]) {
    for (int k = 0; k < 2; k++) {
        RD_CK(s, cudaMemset(s->dCount, 0, sizeof(int)));
        char *items = k ? s->mCur : s->pCur;
        int stride = k ? (int)sizeof(sc_metabolic_particle) : (int)sizeof(sc_particle);
        int n = k ? s->Nm : s->N;
        if (launch(s, "ref_count_nonfinite", n, {&items, &stride, &n, &s->dCount}) || sync(s)) return -1;
        int c = 0;
        RD_CK(s, cudaMemcpy(&c, s->dCount, sizeof(int), cudaMemcpyDeviceToHost));
        out[k] = c;
    }
    return 0;
}

// Names and byte offsets (from the buffer start; negative: before it) of the
// non-zero 4-byte words found in the guards, up to cap entries; returns the
// total found.
int refdev_guards(refdev_sim *s, char *names, int name_len, int64_t *offsets, int cap) {
    int found = 0;
    std::vector<uint32_t> g(kGuardBytes / 4);
    for (auto &kv : s->guards) {
        for (int side = 0; side < 2; side++) {
            const char *src = side ? kv.second.base + kGuardBytes + kv.second.bytes : kv.second.base;
            RD_CK(s, cudaMemcpy(g.data(), src, kGuardBytes, cudaMemcpyDeviceToHost));
            for (size_t w = 0; w < g.size(); w++) {
                if (!g[w]) continue;
                if (found < cap) {
                    strncpy(names + (size_t)found * name_len, kv.first.c_str(), (size_t)name_len - 1);
                    names[(size_t)found * name_len + name_len - 1] = 0;
                    offsets[found] = side ? (int64_t)(kv.second.bytes + w * 4) : -(int64_t)(kGuardBytes - w * 4);
                }
                found++;
            }
        }
    }
    return found;
}

}  // extern "C"
