// sc_ref_device_prelude.h -- force-included (nvcc -include) when the
// reference's own kernel headers (spatial_cell_sim/src/*.cuh, read in place)
// are compiled for sm_103a into oracle/_ref/ref_step.cubin.  TEST
// INFRASTRUCTURE ONLY: that cubin is the reference's CUDA step, which the
// tests compare the product with on the GPU and the bench times beside it.
//
// It supplies what CUDA-samples' helper_math.h, cuRAND and the reference's
// vendored cudaNoise gave the reference, with the same definitions the host
// build of the reference uses (shim/sc_ref_prelude.h), so the device and the
// host builds of the reference compute the same bits:
//   * float3 / float4 are the project's sc_f3 / sc_f4 (layout-identical to
//     CUDA's: 12 bytes, and 16 bytes aligned to 16) with helper_math's
//     component-wise operators (scmath.h); CUDA's own vector types are
//     renamed away after the CUDA headers are in;
//   * sinf / cosf / acosf / powf of float arguments in kernels are
//     scmath.h's functions (the same ones the product's kernels call);
//   * curandState draws from Philox keyed by (seed, particle id, step)
//     (shim_dev/curand_kernel.h);
//   * cudaNoise::simplexNoise, reached only from random_rotation(float3,
//     float, int), which no step kernel calls, is a stub.
// CUDA's real headers, CUB and cuda_fp16.h's __half are used as they are.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cub/cub.cuh>

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

typedef signed char __int8;

// ---- vector types ----------------------------------------------------------
#define float3 sc_f3
#define float4 sc_f4
#define make_float3 sc_make_f3
#define make_float4 sc_make_f4
static __host__ __device__ __forceinline__ float clamp(float f, float a, float b) { return sc_clampf(f, a, b); }

// ---- transcendental functions of the kernels --------------------------------
static __host__ __device__ __forceinline__ float sc_ref_sin(float x) { return sc_sinf(x); }
static __host__ __device__ __forceinline__ double sc_ref_sin(double x) { return ::sin(x); }
static __host__ __device__ __forceinline__ float sc_ref_cos(float x) { return sc_cosf(x); }
static __host__ __device__ __forceinline__ double sc_ref_cos(double x) { return ::cos(x); }
static __host__ __device__ __forceinline__ float sc_ref_acos(float x) { return sc_acosf(x); }
static __host__ __device__ __forceinline__ double sc_ref_acos(double x) { return ::acos(x); }
static __host__ __device__ __forceinline__ float sc_ref_pow(float x, float y) { return sc_powf(x, y); }
static __host__ __device__ __forceinline__ double sc_ref_pow(double x, double y) { return ::pow(x, y); }
#define sin(x) sc_ref_sin(x)
#define cos(x) sc_ref_cos(x)
#define acos(x) sc_ref_acos(x)
#define pow(x, y) sc_ref_pow(x, y)

// ---- cudaNoise (spatial_cell_sim/deps/cudaNoise): not on the step's path -----
#define cudanoise_cuh
namespace cudaNoise {
static __device__ __forceinline__ float simplexNoise(float3, float, int) { return 0.0f; }
}

#include "curand_kernel.h"
#include "json/json.h"
