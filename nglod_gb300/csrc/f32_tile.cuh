// The first layer of the float32 decoder on the tensor cores, shared by the
// float32 query, the fused float32 tracer and the training forward: the
// point-tile and weight-tile formats, the staging of one LOD's decoder, the
// rows of one point tile and the split-TF32 products (tf32_tile.cuh).
#pragma once

#include "dense_common.cuh"
#include "tf32_tile.cuh"

namespace nglod {
namespace f32tile {
constexpr int kTP = 128;     // points per tile (UMMA M)
constexpr int kH = 128;      // hidden units (UMMA N)
constexpr int kK = 32;       // feature channels along K
constexpr int kKC = kK / 4;  // 16-byte core-matrix columns
// A point tile holds the first layer's whole input as TF32 parts: the 32
// summed features, big and small, each a 128 x 32 K-major tile in the
// 128-byte swizzled layout (tile_offset32_sw128: conflict-free row stores
// without padding), and a 128 x 8 position tile [x y z big, 1, x y z small,
// 0].  The weight side (dense K-major) is the feature part big and small and
// two position tiles, [w_xyz big, b0 big, w_xyz big, 0] and [w_xyz small,
// b0 small, 0 ...]: their two products with the position tile add
// p.w + b0 as big*big + small*big + big*small, like the feature part's three
// products, so the first layer lands in TMEM complete.
constexpr uint32_t kTileF = kTP * kK * 4;                 // 16 KB
constexpr uint32_t kTileP = kTP * 8 * 4;                  // 4 KB
constexpr uint32_t kTileA = 2 * kTileF + kTileP;          // one point tile
constexpr uint32_t kWBytes = 2 * kTileF + 2 * kTileP;     // the weight side
static_assert(kTileF % 1024 == 0 && kTileA % 1024 == 0, "swizzled tiles start on 1024-byte boundaries");

// Byte offset of position-tile element (row, k < 8): dense K-major, two
// core-matrix columns.
__host__ __device__ constexpr uint32_t pos_offset(int row, int k) { return tile_offset32(row, k, 2); }
}  // namespace f32tile

// Stages LOD L's decoder for the tensor-core float32 forms at w (the weight
// side of f32tile: feature part big and small, then the two position tiles)
// and w1 (w1 [128]).
__device__ __forceinline__ void stage_tf32_decoder(const nglod_dense_model &m, int L, uint8_t *w, uint8_t *w1, int tid,
                                                   int nthreads) {
    using namespace f32tile;
    const float *w0 = m.w0[L];
    for (int q = tid; q < kH * kKC; q += nthreads) {
        const int j = q / kKC, kc = q % kKC;
        const float *r = w0 + j * 35 + 3 + 4 * kc;
        store_split4(w, w + kTileF, tile_offset32(j, 4 * kc, kKC), make_float4(r[0], r[1], r[2], r[3]));
    }
    for (int j = tid; j < kH; j += nthreads) {
        const float4 u = make_float4(w0[j * 35], w0[j * 35 + 1], w0[j * 35 + 2], m.b0[L][j]);
        const float4 ub = make_float4(tf32_big(u.x), tf32_big(u.y), tf32_big(u.z), tf32_big(u.w));
        uint8_t *pa = w + 2 * kTileF, *pb = pa + kTileP;
        *reinterpret_cast<float4 *>(pa + pos_offset(j, 0)) = ub;
        *reinterpret_cast<float4 *>(pa + pos_offset(j, 4)) = make_float4(ub.x, ub.y, ub.z, 0.f);
        *reinterpret_cast<float4 *>(pb + pos_offset(j, 0)) = make_float4(u.x - ub.x, u.y - ub.y, u.z - ub.z, u.w - ub.w);
        *reinterpret_cast<float4 *>(pb + pos_offset(j, 4)) = make_float4(0.f, 0.f, 0.f, 0.f);
        reinterpret_cast<float *>(w1)[j] = m.w1[L][j];
    }
}

// The rows of one point tile from a warp's cooperative LOD sums (lane holds
// channels 4 (lane % 8) .. +3 of row row0 + 4 p + lane / 8 in acc[p]) and
// from this thread's own point (row row0 + lane).
__device__ __forceinline__ void store_point_rows(uint8_t *tile, int row0, int lane, const float4 (&acc)[8], float px,
                                                 float py, float pz) {
    using namespace f32tile;
#pragma unroll
    for (int p = 0; p < 8; ++p)
        store_split4(tile, tile + kTileF, tile_offset32_sw128(row0 + 4 * p + (lane >> 3), 4 * (lane & 7)), acc[p]);
    const float bx = tf32_big(px), by = tf32_big(py), bz = tf32_big(pz);
    uint8_t *pt = tile + 2 * kTileF;
    *reinterpret_cast<float4 *>(pt + pos_offset(row0 + lane, 0)) = make_float4(bx, by, bz, 1.f);
    *reinterpret_cast<float4 *>(pt + pos_offset(row0 + lane, 4)) = make_float4(px - bx, py - by, pz - bz, 0.f);
}

// The first layer of one point tile (shared address a) against the staged
// weights (shared address w) into TMEM columns d: the feature part's
// big*big + big*small + small*big over K = 32 (four K steps of eight, 32
// bytes along the swizzled line), then the two position products.
__device__ __forceinline__ void issue_first_layer(uint32_t d, uint32_t a, uint32_t w) {
    using namespace f32tile;
    constexpr uint32_t idesc = idesc_tf32_f32(kTP, kH);
    const uint64_t ab = smem_desc_sw128(a), as = smem_desc_sw128(a + kTileF);
    const uint64_t wb = tc::smem_desc(w, 128, kKC * 128), ws = tc::smem_desc(w + kTileF, 128, kKC * 128);
#pragma unroll
    for (int t = 0; t < 3; ++t)
#pragma unroll
        for (int ks = 0; ks < kK / 8; ++ks)
            mma_tf32(d, (t == 2 ? as : ab) + (uint64_t)(ks * 2), (t == 1 ? ws : wb) + (uint64_t)(ks * 16), idesc,
                     (t > 0 || ks > 0) ? 1u : 0u);
    const uint64_t ap = tc::smem_desc(a + 2 * kTileF, 128, 256);
    mma_tf32(d, ap, tc::smem_desc(w + 2 * kTileF, 128, 256), idesc, 1u);
    mma_tf32(d, ap, tc::smem_desc(w + 2 * kTileF + kTileP, 128, 256), idesc, 1u);
}

}  // namespace nglod
