/*
 * Stand-in for the CUDA samples' helper_math.h, which the image does not
 * ship, written for compiling the reference's SPC sources unchanged
 * (sol-renderer/include/spc/spc/spc_math.h:26 includes it).  The traversal
 * kernels use only float * float3; the other operators complete the set.
 * Each is one IEEE operation per component, so the compiled reference
 * arithmetic does not depend on this file beyond that.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/ref_build.py).
 */
#pragma once
#include <cuda_runtime.h>

static __inline__ __host__ __device__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
static __inline__ __host__ __device__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
static __inline__ __host__ __device__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
static __inline__ __host__ __device__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
