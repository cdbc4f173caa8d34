// Float32 products on the tensor cores as tcgen05 kind::tf32 MMAs over
// big / small splits of both operands: x = big + small, big = x with its low
// 13 mantissa bits cleared (a TF32 value), small = x - big (exact);
// a*b ~ ab*bb + ab*bs + as*bb with a relative error of about 2^-21, the size
// of float32's own rounding in a short dot product.  Operands are K-major,
// no-swizzle tiles of 32-bit elements: a core matrix is 8 rows x 16 bytes
// (4 elements along K), 128 contiguous bytes.
#pragma once

#include <stdint.h>

#include "tc_common.cuh"

namespace nglod {

// Byte offset of 32-bit element (row, k) in a K-major tile with kc
// 16-byte core-matrix columns.
__host__ __device__ constexpr uint32_t tile_offset32(int row, int k, int kc) {
    return (uint32_t)(((row / 8) * kc + k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4);
}

__device__ __forceinline__ float tf32_big(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// Stores the big and small parts of four consecutive K elements of one row.
__device__ __forceinline__ void store_split4(uint8_t *big, uint8_t *small, uint32_t off, float4 v) {
    const float4 b = make_float4(tf32_big(v.x), tf32_big(v.y), tf32_big(v.z), tf32_big(v.w));
    *reinterpret_cast<float4 *>(big + off) = b;
    *reinterpret_cast<float4 *>(small + off) = make_float4(v.x - b.x, v.y - b.y, v.z - b.z, v.w - b.w);
}

// D[tmem] (+)= A[smem] * B[smem]^T, one M x N x 8 tf32 step.
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// Instruction descriptor of tcgen05.mma.kind::tf32: D f32 (bits 4-5 = 1),
// A and B tf32 (bits 7-9, 10-12 = 2), both K-major, N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32_f32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

}  // namespace nglod
