// The BF16 decoder tile shared by the dense and sparse tensor-core kernels:
// 128 points x 48 bf16 K columns (A, built by the block) against the
// prepacked 128 hidden x 48 decoder tile (B), fp32 accumulators in 128 TMEM
// columns, and the fp32 epilogue (ReLU, 128 -> 1 layer) on the TMEM rows.
// K order of a point's row: 32 summed features, x y z rounded to bf16, the
// bf16 remainders of x y z, two 1.0 columns against the bf16 split of b0,
// eight zero columns.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"
#include "tc_common.cuh"

namespace nglod {

constexpr int kTP = 128;                 // points per tile = threads per block = UMMA M
constexpr int kHid = 128;                // hidden units = UMMA N
constexpr int kTK = 48;                  // tile K (3 steps of 16)
constexpr int kKC = kTK / 8;             // core-matrix columns along K
constexpr uint32_t kTileBytes = kTP * kTK * 2;
constexpr uint32_t kLbo = 128, kSbo = kKC * 128;
constexpr uint32_t kWaitPolls = 1u << 22;

// Point tiles (A) put their K-adjacent core matrices 160 B apart (the
// descriptor's LBO) instead of 128 B: the quarter warps of the tile writers
// (two rows x four 16-byte pieces, or four rows x two) then store into eight
// different bank groups (at 128 B they would share two or four).  The
// decoder tile (B, packed on the host) keeps the dense layout.
constexpr uint32_t kLboA = 160, kSboA = kKC * kLboA;  // 960 B per 8-row group
constexpr uint32_t kTileBytesA = (kTP / 8) * kSboA;   // 15 KB
__host__ __device__ constexpr uint32_t tile_offset_a(int row, int k) {
    return (uint32_t)((row / 8) * kSboA + (k / 8) * kLboA + (row % 8) * 16 + (k % 8) * 2);
}

// Dynamic shared memory: A tile | B tile | b0[128] | w1[128] | mbarrier |
// TMEM slot | abort flag, padded so that at most four blocks share an SM
// (four x 128 TMEM columns fill the SM's 512).
constexpr size_t kSmemA = 0;
constexpr size_t kSmemB = kSmemA + kTileBytesA;
constexpr size_t kSmemB0 = kSmemB + kTileBytes;
constexpr size_t kSmemW1 = kSmemB0 + kHid * 4;
constexpr size_t kSmemBar = kSmemW1 + kHid * 4;
constexpr size_t kSmemSlot = kSmemBar + 8;
constexpr size_t kSmemAbort = kSmemSlot + 4;
constexpr size_t kSmemBytes = 48 * 1024;

constexpr uint32_t kOneOne = 0x3F803F80u;  // two bf16 1.0: the b0 columns' inputs


__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a in the low half
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Row columns 32..39 of a point: positions as bf16 hi + lo and the 1.0
// columns of the b0 split.
__device__ __forceinline__ uint4 position_columns(float px, float py, float pz) {
    const float hx = __bfloat162float(__float2bfloat16_rn(px));
    const float hy = __bfloat162float(__float2bfloat16_rn(py));
    const float hz = __bfloat162float(__float2bfloat16_rn(pz));
    return make_uint4(pack_bf16x2(hx, hy), pack_bf16x2(hz, px - hx), pack_bf16x2(py - hy, pz - hz), kOneOne);
}

// Second decoder layer on this thread's TMEM row (b0 already inside the
// product): sum_j w1[j] * relu(h[j]), two hidden units per packed FMA.
__device__ __forceinline__ float relu_dot_w1(uint32_t taddr, const float *__restrict__ sw1) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int c = 0; c < kHid / 32; ++c) {
        float v[32];
        tc::tmem_load32(taddr + (uint32_t)(c * 32), v);
        const float2 *w2 = reinterpret_cast<const float2 *>(sw1 + c * 32);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            acc = __ffma2_rn(w2[j], make_float2(fmaxf(v[2 * j], 0.f), fmaxf(v[2 * j + 1], 0.f)), acc);
    }
    return acc.x + acc.y;
}

// 32 bytes of bf16 pairs: the two x corners of 8 channels side by side.
struct alignas(32) PairUnit {
    uint32_t w[8];
};

// 256-bit read-only load (sm_100+); the arrays read this way are 32-byte
// aligned.
__device__ __forceinline__ PairUnit ld_pair_unit(const PairUnit *p) {
    PairUnit r;
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]), "=r"(r.w[4]), "=r"(r.w[5]), "=r"(r.w[6]),
          "=r"(r.w[7])
        : "l"(p));
    return r;
}

// Persistent tracers publish one query point per thread after the fixed
// layout above.
constexpr size_t kSmemQ = (kSmemAbort + 4 + 15) & ~(size_t)15;  // float4 query points [128], 16-byte aligned
static_assert(kSmemQ % 16 == 0 && kSmemQ + kTP * 16 <= kSmemBytes, "query-point array layout");
static_assert(kSmemBar % 8 == 0 && kSmemB % 16 == 0 && kSmemQ + kTP * 16 <= kSmemBytes, "barrier / tile alignment");


}  // namespace nglod
