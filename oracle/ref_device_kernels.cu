// ref_device_kernels.cu -- TEST INFRASTRUCTURE ONLY (oracle).
//
// The reference's own step kernels (spatial_cell_sim/src/{grid,dynamics,
// interactions,metabolites}.cuh, unmodified, read in place from the
// reference tree) compiled for sm_103a into oracle/_ref/ref_step.cubin,
// with shim_dev/sc_ref_device_prelude.h standing in for helper_math,
// cuRAND and cudaNoise.  oracle/ref_device.cu loads the cubin on the GPU
// and replays main.cu's launch sequence with the CUDA toolkit's CUB sort,
// so the reference's CUDA step runs on the GB300 as the reference runs it:
// whole 256/304-byte structs per thread, 256 threads per block, a memset
// of the next buffer before every double-buffered kernel, host
// synchronisations and active-count read-backs where main.cu has them.
//
// Every reference kernel is compiled as a __device__ function (its
// __global__ qualifier is redefined while the reference headers are read)
// and launched through an extern "C" __global__ wrapper of the same
// parameters, which gives the kernels names the host side can look up in
// the cubin without C++ name mangling.  The wrappers add nothing to the
// kernels' work.
#include "types.cuh"
#include "constants.cuh"
#include "config.cuh"
#include "macros.cuh"
#include "math.cuh"
// memory.cuh's DoubleBuffer / DeviceOnlyDoubleBuffer templates rely on MSVC's
// lookup rules (base-class members used unqualified, the injected base name
// without template arguments, memory.cuh:144,151,156,193,200).  Nothing here
// instantiates them; these two spellings only let the front end parse them.
static void *d_Current;
static size_t size;
#define SingleBuffer(x) SingleBuffer<T>(x)
#define DeviceOnlySingleBuffer(x) DeviceOnlySingleBuffer<T>(x)
#include "memory.cuh"
#undef SingleBuffer
#undef DeviceOnlySingleBuffer
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "grid.cuh"
#include "chemistry.cuh"
#include "interactions.cuh"
#include "dynamics.cuh"
#include "metabolites.cuh"
#pragma pop_macro("__global__")

static_assert(sizeof(Particle) == 256, "Particle layout");
static_assert(sizeof(MetabolicParticle) == 304, "MetabolicParticle layout");
static_assert(sizeof(ReducedParticle) == 36, "ReducedParticle layout");
static_assert(sizeof(ReducedMetabolicParticle) == 44, "ReducedMetabolicParticle layout");
static_assert(sizeof(ParticleInteractionInfo) == 96, "ParticleInteractionInfo layout");
static_assert(sizeof(MinimalParticleTypeInfo) == 8, "MinimalParticleTypeInfo layout");
static_assert(offsetof(Particle, pos) == 28 && offsetof(Particle, debugVector) == 240, "Particle layout");
static_assert(offsetof(MetabolicParticle, metabolites) == 256, "MetabolicParticle layout");

// Sizes the host side checks against its own view of the layouts.
extern "C" __device__ const int ref_layout[8] = {
    (int)sizeof(Particle), (int)sizeof(MetabolicParticle), (int)sizeof(ReducedParticle),
    (int)sizeof(ReducedMetabolicParticle), (int)sizeof(ParticleInteractionInfo), (int)sizeof(MinimalParticleTypeInfo),
    (int)sizeof(Config), (int)sizeof(curandState)};

typedef MetabolicParticle MP;
typedef ParticleInteractionInfo PII;
typedef MinimalParticleTypeInfo MPTI;

// ---- the reference's kernels, one wrapper each ------------------------------
extern "C" {
__global__ void ref_updateIndices_P(const Particle *c, unsigned *idx, const int n) { updateIndices<Particle>(c, idx, n); }
__global__ void ref_updateIndices_M(const MP *c, unsigned *idx, const int n) { updateIndices<MP>(c, idx, n); }
__global__ void ref_updateGridRanges(const unsigned *idx, unsigned *ranges, const int n) { updateGridRanges(idx, ranges, n); }
__global__ void ref_move(const int step, curandState *rng, const Particle *c, Particle *x, int n, int *na, int *la,
                         int *ni, unsigned *ranges) { move(step, rng, c, x, n, na, la, ni, ranges); }
__global__ void ref_brownian_P(const int step, curandState *rng, Particle *p, const int n, const float scale) {
    brownianMovementAndRotation<Particle>(step, rng, p, n, scale);
}
__global__ void ref_brownian_M(const int step, curandState *rng, MP *p, const int n, const float scale) {
    brownianMovementAndRotation<MP>(step, rng, p, n, scale);
}
__global__ void ref_moveMetabolicParticles(const int step, curandState *rng, const MP *c, MP *x, int n, unsigned *ranges) {
    moveMetabolicParticles(step, rng, c, x, n, ranges);
}
__global__ void ref_coordinateNoise(const int step, curandState *rng, const Particle *c, Particle *x, int n,
                                    unsigned *ranges, float frac) { coordinateNoise(step, rng, c, x, n, ranges, frac); }
__global__ void ref_applyNoise_P(const int step, curandState *rng, Particle *p, const int n) { applyNoise<Particle>(step, rng, p, n); }
__global__ void ref_applyNoise_M(const int step, curandState *rng, MP *p, const int n) { applyNoise<MP>(step, rng, p, n); }
__global__ void ref_relax(const int step, curandState *rng, const Particle *c, Particle *x, int n, unsigned *ranges,
                          PII *flat) { relax(step, rng, c, x, n, ranges, flat); }
__global__ void ref_relaxMetabolicParticles(const int step, curandState *rng, const MP *c, MP *x, int n, unsigned *mranges,
                                            const Particle *p, unsigned *ranges) {
    relaxMetabolicParticles(step, rng, c, x, n, mranges, p, ranges);
}
__global__ void ref_relaxMetabolicParticlePartners(const int step, curandState *rng, const Particle *c, Particle *x, int n,
                                                   unsigned *ranges, const MP *m, unsigned *mranges) {
    relaxMetabolicParticlePartners(step, rng, c, x, n, ranges, m, mranges);
}
__global__ void ref_applyVelocities_P(const int step, curandState *rng, Particle *p, int n, float f) {
    applyVelocities<Particle>(step, rng, p, n, f);
}
__global__ void ref_applyVelocities_M(const int step, curandState *rng, MP *p, int n, float f) {
    applyVelocities<MP>(step, rng, p, n, f);
}
__global__ void ref_complexify(const int step, curandState *rng, const Particle *c, Particle *x, int n, unsigned *ranges,
                               PII *flat, int *pidx, PII *prules) {
    complexify(step, rng, c, x, n, ranges, flat, pidx, prules);
}
__global__ void ref_transitionInteractions(const int step, curandState *rng, const Particle *c, Particle *x, int n,
                                           int *na, int *la, int *ni, unsigned *ranges, MPTI *types, PII *flat,
                                           int *pidx, PII *prules) {
    transitionInteractions(step, rng, c, x, n, na, la, ni, ranges, types, flat, pidx, prules);
}
__global__ void ref_polymerize(const int step, curandState *rng, Particle *p, int n, int *na, int *la, int *ni,
                               unsigned *ranges, MPTI *types, PII *flat, int *pidx, PII *prules) {
    polymerize(step, rng, p, n, na, la, ni, ranges, types, flat, pidx, prules);
}
__global__ void ref_diffuseMetabolites(const int step, curandState *rng, const MP *c, MP *x, int n, unsigned *ranges) {
    diffuseMetabolites(step, rng, c, x, n, ranges);
}
__global__ void ref_removeInterferingMetabolicParticles(const MP *c, MP *x, int n, unsigned *mranges, const Particle *p,
                                                        unsigned *ranges) {
    removeInterferingMetabolicParticles(c, x, n, mranges, p, ranges);
}
__global__ void ref_reduce_P(const Particle *p, ReducedParticle *r, int n) { reduceParticles<Particle, ReducedParticle>(p, r, n); }
__global__ void ref_reduce_M(const MP *p, ReducedMetabolicParticle *r, int n) {
    reduceParticles<MP, ReducedMetabolicParticle>(p, r, n);
}

// ---- harness kernels (not the reference's) -----------------------------------
// The Philox counter position of every slot before a Brownian kernel: keyed
// by the id of the item in the slot, so the draws follow the item, not the
// slot (the reference seeds XORWOW per slot, main.cu:54-66).
__global__ void ref_set_rng(curandState *st, const char *items, int stride, int n, unsigned long long seed, int step,
                            unsigned su, unsigned sn) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Particle *p = (const Particle *)(items + (size_t)stride * i);
    curandState s;
    s.seed = seed;
    s.id = (uint32_t)p->id;
    s.step = (uint32_t)step;
    s.stream_uniform = su;
    s.stream_normal = sn;
    s.n_uniform = 0;
    s.n_normal = 0;
    st[i] = s;
}
// Active items with a non-finite position (the reference's walled box can
// produce NaN at high density; the harness stops before stepping such a state).
__global__ void ref_count_nonfinite(const char *items, int stride, int n, int *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Particle *p = (const Particle *)(items + (size_t)stride * i);
    if ((p->flags & PARTICLE_FLAG_ACTIVE) &&
        !(sc_isfinitef(p->pos.x) && sc_isfinitef(p->pos.y) && sc_isfinitef(p->pos.z)))
        atomicAdd(out, 1);
}
}  // extern "C"
