// sc_ref_prelude.h -- force-included (g++ -include) when the reference's own
// kernel headers (spatial_cell_sim/src/*.cuh) are compiled as host C++ for
// the oracle in oracle/_ref.  TEST INFRASTRUCTURE ONLY.
//
// It supplies what nvcc, CUDA-samples' helper_math.h, cuRAND, CUB and jsoncpp
// gave the reference:
//   * CUDA qualifiers become plain C++; threadIdx/blockIdx/blockDim are host
//     globals that the harness sets while it runs a kernel body once per
//     thread index (grid emulation);
//   * float3/float4 are the project's sc_f3/sc_f4 with helper_math operator
//     semantics (scmath.h);
//   * CUDA's mixed-type min/max overloads (math_functions.hpp semantics);
//   * sinf/cosf/acosf/powf inside kernels resolve to scmath.h's functions
//     (the same ones the sm_103a step uses) while g_sc_device_math is set,
//     and to the host libm otherwise (host-side setup code);
//   * curandState draws from Philox keyed by (seed, particle id, step), which
//     the harness writes into each slot's state before a Brownian kernel;
//   * __half is binary16 with round-to-nearest-even conversion.
#pragma once

#include <math.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <unordered_map>
#include <functional>
#include <random>
#include <future>
#include <fstream>
#include <iostream>
#include <chrono>
#include <ratio>
#include <ctime>
#include <algorithm>
#include <utility>
#include <stdint.h>

#include "scmath.h"

// ---- qualifiers -----------------------------------------------------------
#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__ static
#define __inline__ inline
#define __forceinline__ inline

typedef signed char __int8;

// ---- vector types ----------------------------------------------------------
typedef sc_f3 float3;
typedef sc_f4 float4;
static inline float3 make_float3(float x, float y, float z) { return sc_make_f3(x, y, z); }
static inline float4 make_float4(float x, float y, float z, float w) { return sc_make_f4(x, y, z, w); }
static inline float clamp(float f, float a, float b) { return sc_clampf(f, a, b); }

struct sc_dim3 { unsigned int x, y, z; };
extern sc_dim3 threadIdx, blockIdx, blockDim, gridDim;

// ---- CUDA's min/max overload set (math_functions.hpp) ----------------------
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
static inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
static inline unsigned int min(int a, unsigned int b) { return min((unsigned int)a, b); }
static inline unsigned int max(int a, unsigned int b) { return max((unsigned int)a, b); }
static inline unsigned int min(unsigned int a, int b) { return min(a, (unsigned int)b); }
static inline unsigned int max(unsigned int a, int b) { return max(a, (unsigned int)b); }
static inline float min(float a, float b) { return fminf(a, b); }
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline double min(double a, double b) { return fmin(a, b); }
static inline double max(double a, double b) { return fmax(a, b); }
static inline double min(float a, double b) { return fmin((double)a, b); }
static inline double max(float a, double b) { return fmax((double)a, b); }
static inline double min(double a, float b) { return fmin(a, (double)b); }
static inline double max(double a, float b) { return fmax(a, (double)b); }

// float overloads of the C math functions, as CUDA declares them globally
using std::fabs;
using std::sqrt;
using std::ceil;

// ---- transcendental functions of the kernels --------------------------------
extern bool g_sc_device_math;
static inline float sc_ref_sin(float x) { return g_sc_device_math ? sc_sinf(x) : ::sinf(x); }
static inline double sc_ref_sin(double x) { return ::sin(x); }
static inline float sc_ref_cos(float x) { return g_sc_device_math ? sc_cosf(x) : ::cosf(x); }
static inline double sc_ref_cos(double x) { return ::cos(x); }
static inline float sc_ref_acos(float x) { return g_sc_device_math ? sc_acosf(x) : ::acosf(x); }
static inline double sc_ref_acos(double x) { return ::acos(x); }
static inline float sc_ref_pow(float x, float y) { return g_sc_device_math ? sc_powf(x, y) : ::powf(x, y); }
static inline double sc_ref_pow(double x, double y) { return ::pow(x, y); }
#define sin(x) sc_ref_sin(x)
#define cos(x) sc_ref_cos(x)
#define acos(x) sc_ref_acos(x)
#define pow(x, y) sc_ref_pow(x, y)

// ---- atomics (the harness runs thread indices one after another) ----------
static inline int atomicAdd(int *p, int v) { int old = *p; *p = old + v; return old; }

// ---- runtime API used by memory.cuh / grid.cuh -------------------------------
typedef int cudaError_t;
#define cudaSuccess 0
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
static inline cudaError_t cudaMalloc(void **p, size_t n) { *p = calloc(n ? n : 1, 1); return *p ? 0 : 2; }
template <typename T> static inline cudaError_t cudaMalloc(T **p, size_t n) { return cudaMalloc((void **)p, n); }
static inline cudaError_t cudaFree(void *p) { free(p); return 0; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return 0; }
static inline cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return 0; }
static inline cudaError_t cudaDeviceSynchronize() { return 0; }
static inline cudaError_t cudaGetLastError() { return 0; }
static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }

// ---- cuda_fp16.h --------------------------------------------------------------
struct __half {
    uint16_t bits;
    __half() : bits(0) {}
    __half(float f) : bits(sc_f2h(f)) {}
};

// ---- cudaNoise (spatial_cell_sim/deps/cudaNoise): only reached from
// random_rotation(float3, float, int), which the step never calls -------------
#define cudanoise_cuh
namespace cudaNoise { float simplexNoise(float3 pos, float scale, int seed); }

#include "curand_kernel.h"
#include "cub/cub.cuh"
#include "json/json.h"
