// Device stand-in for curand_kernel.h (oracle only; the device build of the
// reference).  As in the host build (shim/curand_kernel.h) a state is a
// Philox counter position {seed, particle id, step, streams, draws}: the
// harness writes it for every slot before a Brownian kernel, and uniform /
// normal draws advance separate counters.
#pragma once
#include "scmath.h"

struct curandState {
    uint64_t seed;
    uint32_t id;
    uint32_t step;
    uint32_t stream_uniform;
    uint32_t stream_normal;
    uint32_t n_uniform;
    uint32_t n_normal;
};

static __host__ __device__ __forceinline__ void curand_init(unsigned long long seed, unsigned long long,
                                                            unsigned long long, curandState *s) {
    s->seed = seed; s->id = 0; s->step = 0;
    s->stream_uniform = SC_STREAM_P_UNIFORM; s->stream_normal = SC_STREAM_P_NORMAL;
    s->n_uniform = 0; s->n_normal = 0;
}
static __host__ __device__ __forceinline__ float curand_uniform(curandState *s) {
    return sc_uniform(s->seed, s->stream_uniform, s->id, s->step, s->n_uniform++);
}
static __host__ __device__ __forceinline__ float curand_normal(curandState *s) {
    return sc_normal(s->seed, s->stream_normal, s->id, s->step, s->n_normal++);
}
