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

// Byte offset of 32-bit element (row, k < 32) in a K-major tile stored in
// the 128-byte swizzled layout: each row is one 128-byte line, eight rows
// form a 1024-byte atom, and the 16-byte piece k / 4 of row r sits at piece
// (k / 4) ^ (r % 8) of its line.  The tile must start on a 1024-byte
// boundary.  The eight pieces of one row land in eight different bank
// groups, and no padding is needed.
__host__ __device__ constexpr uint32_t tile_offset32_sw128(int row, int k) {
    return (uint32_t)((row / 8) * 1024 + (row % 8) * 128 + ((((k / 4) ^ (row % 8)) & 7) * 16) + (k % 4) * 4);
}

// Shared-memory descriptor of a K-major 128-byte swizzled tile (layout type
// 2 in bits 61-63; 1024 bytes between 8-row atoms; the leading offset is
// unused by this layout).  A K step inside the 128-byte line advances the
// start address.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    return tc::smem_desc(saddr, 16, 1024) | ((uint64_t)2 << 61);
}

// Second decoder layer on this thread's TMEM row of 128 fp32 columns (the
// whole first layer, biases included, already in the product):
// sum_j w1[j] * relu(h[j]), two hidden units per packed FMA.
__device__ __forceinline__ float relu_dot_w1_f32(uint32_t taddr, const float *__restrict__ sw1) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        float v[32];
        tc::tmem_load32(taddr + (uint32_t)(c * 32), v);
        const float2 *w2 = reinterpret_cast<const float2 *>(sw1 + c * 32);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            acc = __ffma2_rn(w2[j], make_float2(fmaxf(v[2 * j], 0.f), fmaxf(v[2 * j + 1], 0.f)), acc);
    }
    return acc.x + acc.y;
}

// Instruction descriptor of tcgen05.mma.kind::tf32: D f32 (bits 4-5 = 1),
// A and B tf32 (bits 7-9, 10-12 = 2), both K-major, N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32_f32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

}  // namespace nglod
