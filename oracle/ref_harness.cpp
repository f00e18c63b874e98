// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (oracle).
//
// Builds the reference's own step (spatial_cell_sim/src/{grid,dynamics,
// interactions,metabolites}.cuh) for the host CPU, unmodified and read in
// place from the reference tree, with shim/sc_ref_prelude.h standing in for
// nvcc, cuRAND, CUB, helper_math and jsoncpp.  Every kernel body is run once
// per thread index in ascending order (grid emulation), and the launch
// sequence of one step is main.cu:347-661 (frame persistence excluded),
// including the clearNextOnDevice() memsets before every double-buffered
// kernel.  The result is oracle/_ref/libscref.so, which the tests use to pin
// the CPU restatement (oracle/scport.cpp) and to generate golden vectors.
//
// Deviations from running main.cu on a GPU, all forced by running one
// thread at a time on the host:
//  * curandState is a Philox counter position keyed by (seed, particle id,
//    step) (shim/curand_kernel.h) instead of XORWOW per slot;
//  * transcendental functions in kernels are scmath.h's (the sm_103a build
//    uses the same functions);
//  * CUB's SortPairs is std::stable_sort (same stable order);
//  * thread indices run in ascending order, which fixes the order of the
//    atomicAdd slot/id allocation in polymerize (interactions.cuh:640-642);
//  * the partner-mapped rule list is built in ascending rule id per type
//    (the reference's order is std::unordered_map iteration order,
//    interactions.cuh:91-132, which differs between standard libraries).
#include "types.cuh"
#include "constants.cuh"
#include "config.cuh"
#include "macros.cuh"
#include "math.cuh"
// memory.cuh's DoubleBuffer / DeviceOnlyDoubleBuffer templates rely on MSVC's
// lookup rules (base-class members used unqualified, the injected base name
// without template arguments, memory.cuh:144,151,156,193,200).  The harness
// never instantiates them; these two spellings only let g++ parse them.
static void *d_Current;
static size_t size;
#define SingleBuffer(x) SingleBuffer<T>(x)
#define DeviceOnlySingleBuffer(x) DeviceOnlySingleBuffer<T>(x)
#include "memory.cuh"
#undef SingleBuffer
#undef DeviceOnlySingleBuffer
#include "grid.cuh"
#include "chemistry.cuh"
#include "interactions.cuh"
#include "dynamics.cuh"
#include "metabolites.cuh"

#include <unistd.h>

#include "spatialcell.h"

sc_dim3 threadIdx, blockIdx, blockDim, gridDim;
bool g_sc_device_math = false;

static_assert(sizeof(Particle) == sizeof(sc_particle), "Particle layout");
static_assert(sizeof(MetabolicParticle) == sizeof(sc_metabolic_particle), "MetabolicParticle layout");
static_assert(sizeof(ReducedParticle) == sizeof(sc_reduced_particle), "ReducedParticle layout");
static_assert(sizeof(ReducedMetabolicParticle) == sizeof(sc_reduced_metabolic_particle), "ReducedMetabolicParticle layout");
static_assert(sizeof(ParticleInteractionInfo) == sizeof(sc_rule), "ParticleInteractionInfo layout");
static_assert(offsetof(Particle, debugVector) == 240, "Particle layout");
static_assert(offsetof(ParticleInteractionInfo, relativePosition) == 68, "rule layout");

template <class F>
static void launch(long long nthreads, F kernel) {
    blockDim.x = CUDA_THREADS_PER_BLOCK; blockDim.y = blockDim.z = 1;
    long long blocks = (nthreads + CUDA_THREADS_PER_BLOCK - 1) / CUDA_THREADS_PER_BLOCK;
    gridDim.x = (unsigned)blocks; gridDim.y = gridDim.z = 1;
    threadIdx.y = threadIdx.z = blockIdx.y = blockIdx.z = 0;
    g_sc_device_math = true;
    for (long long b = 0; b < blocks; b++) {
        blockIdx.x = (unsigned)b;
        for (unsigned t = 0; t < CUDA_THREADS_PER_BLOCK; t++) { threadIdx.x = t; kernel(); }
    }
    g_sc_device_math = false;
}

struct oref_sim {
    Config cfg;
    int N = 0, Nm = 0;
    uint64_t seed = 42;
    // one element of slack in front: polymerize's end-of-chain branch can
    // store to particles[-1] (interactions.cuh:728 with prevMonomerIdx == -1)
    Particle *pBase[2] = {nullptr, nullptr};
    Particle *pCur = nullptr, *pNext = nullptr;
    MetabolicParticle *mCur = nullptr, *mNext = nullptr;
    unsigned *keysP = nullptr, *keysP2 = nullptr, *keysM = nullptr, *keysM2 = nullptr;
    unsigned *rangesPBase = nullptr, *rangesMBase = nullptr;  // 16 words of slack in front
    unsigned *rangesP = nullptr, *rangesM = nullptr;
    uint32_t *permP = nullptr, *permM = nullptr;
    curandState *rngP = nullptr, *rngM = nullptr;
    MinimalParticleTypeInfo *types = nullptr; int nTypes = 0;
    ParticleInteractionInfo *flatRules = nullptr; int nFlat = 0;
    int *partnerIndex = nullptr; int nPartnerIndex = 0;
    ParticleInteractionInfo *partnerRules = nullptr;
    int nActive = 0, lastActive = -1, nextId = 0, nActiveM = 0;
    int step = 0;
    size_t cells = 0;
};

static Config make_config(const sc_config *c) {
    char buf[2048];
    snprintf(buf, sizeof buf,
             "{\"numParticles\": %d, \"numMetabolicParticles\": %d, \"steps\": %d, \"simSize\": %.9g,"
             " \"maxInteractionDistance\": %.9g, \"maxDiffusionDistance\": %.9g, \"gridCellSize\": %.9g,"
             " \"movementNoiseScale\": %.9g, \"rotationNoiseScale\": %.9g, \"metaboliteMovementNoiseScale\": %.9g,"
             " \"velocityDecay\": %.9g, \"angularVelocityDecay\": %.9g, \"noiseCoordinationSteps\": %d,"
             " \"relaxationSteps\": %d, \"metaboliteDiffusionSteps\": %d, \"persistEveryNthFrame\": %d,"
             " \"reportEveryNthFrame\": %d}",
             c->num_particles, c->num_metabolic_particles, c->steps, c->sim_size, c->max_interaction_distance,
             c->max_diffusion_distance, c->grid_cell_size, c->movement_noise_scale, c->rotation_noise_scale,
             c->metabolite_movement_noise_scale, c->velocity_decay, c->angular_velocity_decay,
             c->noise_coordination_steps, c->relaxation_steps, c->metabolite_diffusion_steps,
             c->persist_every_nth_frame, c->report_every_nth_frame);
    scjson::Value v;
    std::string err;
    scjson::parse(buf, v, err);
    return Config(Json::Value(v));
}

template <class T>
static void update_grid_and_sort(oref_sim *s, T *&cur, T *&next, unsigned *&keys, unsigned *&keys2,
                                 unsigned *ranges, uint32_t *perm, int n) {
    // grid.cuh:111-139 with CUB's SortPairs replaced by the same stable order
    T *c = cur;
    unsigned *k = keys;
    launch(n, [&] { updateIndices<T>(c, k, n); });
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    for (int i = 0; i < n; i++) {
        keys2[i] = keys[order[i]];
        next[i] = cur[order[i]];
        perm[i] = (uint32_t)order[i];
    }
    std::swap(cur, next);
    std::swap(keys, keys2);
    memset(ranges, 0, s->cells * 2 * sizeof(unsigned));
    unsigned *kk = keys;
    launch((long long)s->cfg.totalGridCells, [&] { updateGridRanges(kk, ranges, n); });
}

static void set_rng(curandState *st, const Particle *items, size_t stride, int n, uint64_t seed, int step,
                    uint32_t su, uint32_t sn) {
    for (int i = 0; i < n; i++) {
        const Particle *p = (const Particle *)((const char *)items + stride * i);
        st[i].seed = seed; st[i].id = (uint32_t)p->id; st[i].step = (uint32_t)step;
        st[i].stream_uniform = su; st[i].stream_normal = sn;
        st[i].n_uniform = 0; st[i].n_normal = 0;
    }
}

extern "C" {

oref_sim *oref_create(const sc_config *c, const sc_type_info *types, int n_types, const sc_rule *rules, int n_rules) {
    oref_sim *s = new oref_sim();
    s->cfg = make_config(c);
    s->N = c->num_particles;
    s->Nm = c->num_metabolic_particles;
    s->seed = c->seed;
    s->cells = (size_t)s->cfg.totalGridCells;
    d_Config = s->cfg;
    s->pBase[0] = (Particle *)calloc((size_t)s->N + 2, sizeof(Particle));
    s->pBase[1] = (Particle *)calloc((size_t)s->N + 2, sizeof(Particle));
    s->pCur = s->pBase[0] + 1;
    s->pNext = s->pBase[1] + 1;
    s->mCur = (MetabolicParticle *)calloc((size_t)s->Nm + 1, sizeof(MetabolicParticle));
    s->mNext = (MetabolicParticle *)calloc((size_t)s->Nm + 1, sizeof(MetabolicParticle));
    s->keysP = (unsigned *)calloc((size_t)s->N + 1, 4); s->keysP2 = (unsigned *)calloc((size_t)s->N + 1, 4);
    s->keysM = (unsigned *)calloc((size_t)s->Nm + 1, 4); s->keysM2 = (unsigned *)calloc((size_t)s->Nm + 1, 4);
    s->rangesPBase = (unsigned *)calloc(s->cells * 2 + 32, 4);
    s->rangesMBase = (unsigned *)calloc(s->cells * 2 + 32, 4);
    s->rangesP = s->rangesPBase + 16;
    s->rangesM = s->rangesMBase + 16;
    s->permP = (uint32_t *)calloc((size_t)s->N + 1, 4);
    s->permM = (uint32_t *)calloc((size_t)s->Nm + 1, 4);
    s->rngP = (curandState *)calloc((size_t)s->N + 1, sizeof(curandState));
    s->rngM = (curandState *)calloc((size_t)s->Nm + 1, sizeof(curandState));
    // tables: id-indexed types, id-indexed rules (first of duplicate ids),
    // partner index sized (maxRuleId + 1) * 2 as in interactions.cuh:118
    s->nTypes = n_types;
    s->types = (MinimalParticleTypeInfo *)calloc((size_t)n_types + 1, sizeof(MinimalParticleTypeInfo));
    for (int i = 0; i < n_types; i++) { s->types[i].radius = types[i].radius; s->types[i].hydrophobic = types[i].hydrophobic; }
    int maxId = 0;
    for (int i = 0; i < n_rules; i++) maxId = std::max(maxId, rules[i].id);
    s->nFlat = maxId + 1;
    s->flatRules = (ParticleInteractionInfo *)calloc((size_t)s->nFlat, sizeof(ParticleInteractionInfo));
    std::vector<char> seen(s->nFlat, 0);
    std::vector<const sc_rule *> uniq;
    for (int i = 0; i < n_rules; i++) {
        int id = rules[i].id;
        if (id < 0 || seen[id]) continue;
        seen[id] = 1;
        memcpy(&s->flatRules[id], &rules[i], sizeof(sc_rule));
    }
    for (int id = 0; id < s->nFlat; id++) if (seen[id]) uniq.push_back((const sc_rule *)&s->flatRules[id]);
    s->nPartnerIndex = s->nFlat * 2;
    s->partnerIndex = (int *)calloc((size_t)s->nPartnerIndex, sizeof(int));
    std::map<int, std::vector<int>> byType;
    for (const sc_rule *r : uniq) {
        if (r->first_partner_type >= 0) byType[r->first_partner_type].push_back(r->id);
        if (r->second_partner_type >= 0) byType[r->second_partner_type].push_back(r->id);
    }
    s->partnerRules = (ParticleInteractionInfo *)calloc(uniq.size() * 2 + 1, sizeof(ParticleInteractionInfo));
    int np = 0;
    for (auto &kv : byType) {
        if (kv.first * 2 + 1 < s->nPartnerIndex) {
            s->partnerIndex[kv.first * 2] = np;
            s->partnerIndex[kv.first * 2 + 1] = np + (int)kv.second.size();
        }
        for (int id : kv.second) s->partnerRules[np++] = s->flatRules[id];
    }
    return s;
}

void oref_destroy(oref_sim *s) {
    if (!s) return;
    free(s->pBase[0]); free(s->pBase[1]); free(s->mCur); free(s->mNext);
    free(s->keysP); free(s->keysP2); free(s->keysM); free(s->keysM2);
    free(s->rangesPBase); free(s->rangesMBase); free(s->permP); free(s->permM);
    free(s->rngP); free(s->rngM); free(s->types); free(s->flatRules); free(s->partnerIndex); free(s->partnerRules);
    delete s;
}

int oref_load_state(oref_sim *s, const sc_particle *p, int n, const sc_metabolic_particle *m, int nm, int step,
                    int next_id) {
    if (n > s->N || nm > s->Nm || n < 0 || nm < 0) return -1;
    memset(s->pCur, 0, (size_t)s->N * sizeof(Particle));
    memset(s->mCur, 0, (size_t)s->Nm * sizeof(MetabolicParticle));
    if (n) memcpy(s->pCur, p, (size_t)n * sizeof(Particle));
    if (nm) memcpy(s->mCur, m, (size_t)nm * sizeof(MetabolicParticle));
    s->nActive = n; s->lastActive = n - 1; s->nextId = next_id; s->nActiveM = nm; s->step = step;
    return 0;
}

// One kernel (or the kernel pair) of main.cu's loop.
int oref_run_phase(oref_sim *s, int phase, int arg) {
    d_Config = s->cfg;
    Config &cfg = s->cfg;
    const int step = s->step;
    switch (phase) {
        case SC_PHASE_SORT_PARTICLES:
            update_grid_and_sort(s, s->pCur, s->pNext, s->keysP, s->keysP2, s->rangesP, s->permP, s->N);
            s->lastActive = s->nActive - 1;   // main.cu:369-371
            break;
        case SC_PHASE_SORT_METABOLIC:
            update_grid_and_sort(s, s->mCur, s->mNext, s->keysM, s->keysM2, s->rangesM, s->permM, s->Nm);
            break;
        case SC_PHASE_MOVE_BROWNIAN: {  // main.cu:375-395
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            int *na = &s->nActive, *la = &s->lastActive, *ni = &s->nextId;
            launch(n, [&] { move(step, s->rngP, c, x, n, na, la, ni, s->rangesP); });
            std::swap(s->pCur, s->pNext);
            set_rng(s->rngP, s->pCur, sizeof(Particle), s->N, s->seed, step, SC_STREAM_P_UNIFORM, SC_STREAM_P_NORMAL);
            Particle *cc = s->pCur;
            float scale = cfg.movementNoiseScale;
            launch(n, [&] { brownianMovementAndRotation<Particle>(step, s->rngP, cc, n, scale); });
            break;
        }
        case SC_PHASE_MOVE_BROWNIAN_METAB: {  // main.cu:402-419
            int n = s->nActiveM;
            memset(s->mNext, 0, (size_t)s->Nm * sizeof(MetabolicParticle));
            MetabolicParticle *c = s->mCur, *x = s->mNext;
            launch(n, [&] { moveMetabolicParticles(step, s->rngM, c, x, n, s->rangesM); });
            std::swap(s->mCur, s->mNext);
            set_rng(s->rngM, s->mCur, sizeof(MetabolicParticle), s->Nm, s->seed, step, SC_STREAM_M_UNIFORM,
                    SC_STREAM_M_NORMAL);
            MetabolicParticle *cc = s->mCur;
            float scale = cfg.metaboliteMovementNoiseScale;
            launch(n, [&] { brownianMovementAndRotation<MetabolicParticle>(step, s->rngM, cc, n, scale); });
            break;
        }
        case SC_PHASE_COORDINATE_NOISE: {  // main.cu:426-441
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            float frac = (float)arg / cfg.noiseCoordinationSteps;
            launch(n, [&] { coordinateNoise(step, s->rngP, c, x, n, s->rangesP, frac); });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_APPLY_NOISE: {  // main.cu:443-455
            int n = s->nActive, nm = s->nActiveM;
            Particle *c = s->pCur;
            MetabolicParticle *mc = s->mCur;
            launch(n, [&] { applyNoise<Particle>(step, s->rngP, c, n); });
            launch(nm, [&] { applyNoise<MetabolicParticle>(step, s->rngM, mc, nm); });
            break;
        }
        case SC_PHASE_RELAX: {  // main.cu:478-496
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            launch(n, [&] { relax(step, s->rngP, c, x, n, s->rangesP, s->flatRules); });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_RELAX_METAB: {  // main.cu:511-523
            int nm = s->nActiveM;
            memset(s->mNext, 0, (size_t)s->Nm * sizeof(MetabolicParticle));
            MetabolicParticle *c = s->mCur, *x = s->mNext;
            Particle *pc = s->pCur;
            launch(nm, [&] { relaxMetabolicParticles(step, s->rngM, c, x, nm, s->rangesM, pc, s->rangesP); });
            std::swap(s->mCur, s->mNext);
            break;
        }
        case SC_PHASE_RELAX_PARTNERS: {  // main.cu:526-537
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            MetabolicParticle *mc = s->mCur;
            launch(n, [&] { relaxMetabolicParticlePartners(step, s->rngP, c, x, n, s->rangesP, mc, s->rangesM); });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_APPLY_VELOCITIES: {  // main.cu:548-561
            int n = s->nActive, nm = s->nActiveM;
            Particle *c = s->pCur;
            MetabolicParticle *mc = s->mCur;
            launch(n, [&] { applyVelocities<Particle>(step, s->rngP, c, n, 0.45f); });
            launch(nm, [&] { applyVelocities<MetabolicParticle>(step, s->rngM, mc, nm, 0.45f); });
            break;
        }
        case SC_PHASE_COMPLEXIFY: {  // main.cu:567-579 (arg: the step argument, -1 at start-up)
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            launch(n, [&] { complexify(arg, s->rngP, c, x, n, s->rangesP, s->flatRules, s->partnerIndex, s->partnerRules); });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_TRANSITION: {  // main.cu:582-598
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            int *na = &s->nActive, *la = &s->lastActive, *ni = &s->nextId;
            launch(n, [&] {
                transitionInteractions(step, s->rngP, c, x, n, na, la, ni, s->rangesP, s->types, s->flatRules,
                                       s->partnerIndex, s->partnerRules);
            });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_POLYMERIZE: {  // main.cu:600-616
            int n = s->nActive;
            Particle *c = s->pCur;
            int *na = &s->nActive, *la = &s->lastActive, *ni = &s->nextId;
            launch(n, [&] {
                polymerize(step, s->rngP, c, n, na, la, ni, s->rangesP, s->types, s->flatRules, s->partnerIndex,
                           s->partnerRules);
            });
            break;
        }
        case SC_PHASE_PROPAGATE_STATE: {  // the launch main.cu:618-631 leaves commented out
            int n = s->nActive;
            memset(s->pNext, 0, (size_t)s->N * sizeof(Particle));
            Particle *c = s->pCur, *x = s->pNext;
            launch(n, [&] {
                propagateState(step, s->rngP, c, x, n, s->rangesP, s->flatRules, s->partnerIndex, s->partnerRules);
            });
            std::swap(s->pCur, s->pNext);
            break;
        }
        case SC_PHASE_DIFFUSE: {  // main.cu:637-649
            int nm = s->nActiveM;
            memset(s->mNext, 0, (size_t)s->Nm * sizeof(MetabolicParticle));
            MetabolicParticle *c = s->mCur, *x = s->mNext;
            launch(nm, [&] { diffuseMetabolites(step, s->rngM, c, x, nm, s->rangesM); });
            std::swap(s->mCur, s->mNext);
            break;
        }
        case SC_PHASE_REMOVE_INTERFERING: {  // main.cu:302-311
            int nm = s->nActiveM;
            memset(s->mNext, 0, (size_t)s->Nm * sizeof(MetabolicParticle));
            MetabolicParticle *c = s->mCur, *x = s->mNext;
            Particle *pc = s->pCur;
            launch(nm, [&] { removeInterferingMetabolicParticles(c, x, nm, s->rangesM, pc, s->rangesP); });
            std::swap(s->mCur, s->mNext);
            break;
        }
        case SC_PHASE_END_STEP:
            s->step++;
            break;
        default:
            return -1;
    }
    return 0;
}

int oref_prepare(oref_sim *s) {  // main.cu:284-338 (frame 0 not written)
    oref_run_phase(s, SC_PHASE_SORT_PARTICLES, 0);
    oref_run_phase(s, SC_PHASE_SORT_METABOLIC, 0);
    oref_run_phase(s, SC_PHASE_REMOVE_INTERFERING, 0);
    oref_run_phase(s, SC_PHASE_COMPLEXIFY, -1);
    return 0;
}

int oref_step(oref_sim *s, int n_steps) {  // main.cu:347-661
    for (int k = 0; k < n_steps; k++) {
        oref_run_phase(s, SC_PHASE_SORT_PARTICLES, 0);
        oref_run_phase(s, SC_PHASE_SORT_METABOLIC, 0);
        oref_run_phase(s, SC_PHASE_MOVE_BROWNIAN, 0);
        oref_run_phase(s, SC_PHASE_MOVE_BROWNIAN_METAB, 0);
        for (int j = 0; j < s->cfg.noiseCoordinationSteps; j++) oref_run_phase(s, SC_PHASE_COORDINATE_NOISE, j);
        oref_run_phase(s, SC_PHASE_APPLY_NOISE, 0);
        for (int j = 0; j < s->cfg.relaxationSteps; j++) {
            oref_run_phase(s, SC_PHASE_RELAX, j);
            if (j % 2 == 0) {
                oref_run_phase(s, SC_PHASE_RELAX_METAB, j);
                oref_run_phase(s, SC_PHASE_RELAX_PARTNERS, j);
            }
        }
        oref_run_phase(s, SC_PHASE_APPLY_VELOCITIES, 0);
        oref_run_phase(s, SC_PHASE_COMPLEXIFY, s->step);
        oref_run_phase(s, SC_PHASE_TRANSITION, 0);
        oref_run_phase(s, SC_PHASE_POLYMERIZE, 0);
        for (int j = 0; j < s->cfg.metaboliteDiffusionSteps; j++) oref_run_phase(s, SC_PHASE_DIFFUSE, j);
        oref_run_phase(s, SC_PHASE_END_STEP, 0);
    }
    return 0;
}

int oref_export_state(oref_sim *s, sc_particle *p, sc_metabolic_particle *m) {
    if (p) memcpy(p, s->pCur, (size_t)s->N * sizeof(Particle));
    if (m) memcpy(m, s->mCur, (size_t)s->Nm * sizeof(MetabolicParticle));
    return 0;
}

int oref_export_grid(oref_sim *s, int which, uint32_t *ranges, uint32_t *perm) {
    if (ranges) memcpy(ranges, which ? s->rangesM : s->rangesP, s->cells * 2 * 4);
    if (perm) memcpy(perm, which ? s->permM : s->permP, (size_t)(which ? s->Nm : s->N) * 4);
    return 0;
}

int oref_get_counters(oref_sim *s, sc_counters *c) {
    memset(c, 0, sizeof *c);
    c->n_active_particles = s->nActive;
    c->n_active_metabolic_particles = s->nActiveM;
    c->next_particle_id = s->nextId;
    c->step = s->step;
    return 0;
}

int oref_reduce_frame(oref_sim *s, sc_reduced_particle *rp, sc_reduced_metabolic_particle *rm) {
    // main.cu:95-126 (clearOnDevice + reduceParticles over the active counters)
    ReducedParticle *rd = (ReducedParticle *)calloc((size_t)s->N + 1, sizeof(ReducedParticle));
    ReducedMetabolicParticle *qd = (ReducedMetabolicParticle *)calloc((size_t)s->Nm + 1, sizeof(ReducedMetabolicParticle));
    int n = s->nActive, nm = s->nActiveM;
    launch(n, [&] { reduceParticles<Particle, ReducedParticle>(s->pCur, rd, n); });
    launch(nm, [&] { reduceParticles<MetabolicParticle, ReducedMetabolicParticle>(s->mCur, qd, nm); });
    if (rp) memcpy(rp, rd, (size_t)s->N * sizeof(ReducedParticle));
    if (rm) memcpy(rm, qd, (size_t)s->Nm * sizeof(ReducedMetabolicParticle));
    free(rd);
    free(qd);
    return 0;
}

// The reference's own table loaders, run on <sim_dir>/../universe-config/gen.
int oref_load_tables(const char *sim_dir, sc_type_info *types, int cap_types, int *n_types, sc_rule *flat_rules,
                     int cap_flat, int *n_flat, int *partner_index, int cap_index, int *n_index,
                     sc_rule *partner_rules, int cap_partner, int *n_partner) {
    char old[4096];
    if (!getcwd(old, sizeof old)) return -1;
    if (chdir(sim_dir) != 0) return -1;
    int rc = 0;
    try {
        auto typeInfo = loadParticleTypeInfo();
        auto flatTypes = flattenParticleTypeInfo(typeInfo);
        *n_types = (int)flatTypes->count;
        for (int i = 0; i < *n_types && i < cap_types; i++) {
            types[i].radius = flatTypes->h_Current[i].radius;
            types[i].hydrophobic = flatTypes->h_Current[i].hydrophobic;
        }
        auto rules = loadComplexificationInfo();
        auto flat = flattenComplexificationInfo(rules);
        *n_flat = (int)flat->count;
        for (int i = 0; i < *n_flat && i < cap_flat; i++) memcpy(&flat_rules[i], &flat->h_Current[i], sizeof(sc_rule));
        auto pm = partnerMapComplexificationInfo(rules);
        *n_index = (int)pm.first->count;
        for (int i = 0; i < *n_index && i < cap_index; i++) partner_index[i] = pm.first->h_Current[i];
        *n_partner = (int)pm.second->count;
        for (int i = 0; i < *n_partner && i < cap_partner; i++)
            memcpy(&partner_rules[i], &pm.second->h_Current[i], sizeof(sc_rule));
        delete flatTypes; delete flat; delete pm.first; delete pm.second; delete typeInfo; delete rules;
    } catch (...) {
        rc = -1;
    }
    if (chdir(old) != 0) rc = -1;
    return rc;
}

// Config(Json::Value) of config.cuh:46-75 on a config.json file.
int oref_load_config(const char *path, sc_config *out, int *n_grid_cells, int *n_grid_bits) {
    std::ifstream f(path);
    if (!f) return -1;
    Json::Value v;
    try { f >> v; } catch (...) { return -1; }
    Config c(v);
    out->num_particles = c.numParticles;
    out->num_metabolic_particles = c.numMetabolicParticles;
    out->steps = c.steps;
    out->sim_size = c.simSize;
    out->max_interaction_distance = c.maxInteractionDistance;
    out->max_diffusion_distance = c.maxDiffusionDistance;
    out->grid_cell_size = c.gridCellSize;
    out->movement_noise_scale = c.movementNoiseScale;
    out->rotation_noise_scale = c.rotationNoiseScale;
    out->metabolite_movement_noise_scale = c.metaboliteMovementNoiseScale;
    out->velocity_decay = c.velocityDecay;
    out->angular_velocity_decay = c.angularVelocityDecay;
    out->noise_coordination_steps = c.noiseCoordinationSteps;
    out->relaxation_steps = c.relaxationSteps;
    out->metabolite_diffusion_steps = c.metaboliteDiffusionSteps;
    out->persist_every_nth_frame = c.persistEveryNthFrame;
    out->report_every_nth_frame = c.reportEveryNthFrame;
    *n_grid_cells = c.nGridCells;
    *n_grid_bits = c.nGridCellsBits;
    return 0;
}

}  // extern "C"
