// BF16 form of the dense path: bf16 channel-last feature volumes gathered
// with 16-byte loads (point queries: each lane computes its own point's
// corner offsets and weights and four lanes per point load the corners, 8
// channels each, or with 32-byte loads from pair volumes that hold each
// vertex beside its +x neighbour; the tracer: two lanes per point, 16
// channels each), the LOD sum kept in fp32 and written as one
// row of a bf16 tile in shared memory, and the decoder's 35 -> 128 layer run
// by tcgen05.mma on 128-point tiles with the accumulator in tensor memory.
// b0, ReLU and the 128 -> 1 layer are an fp32 epilogue on the TMEM rows.
#include <cuda_bf16.h>

#include <algorithm>
#include <string.h>

#include "bf16_tile.cuh"

namespace nglod {

// Corner set of one point in one bf16 volume (s vertices per side) with
// PyTorch grid_sample arithmetic (align_corners, border clamp): the vertex
// index of corner 0 in bits 0..27 and whether the x / y / z neighbour
// differs from it (not clamped) in bits 28..30; the eight trilinear weights
// in tnw..bse order.
__device__ __forceinline__ void corner_set(int s, float px, float py, float pz, uint32_t &packed, float (&w)[8]) {
    const float sm1 = (float)(s - 1);
    const float ix = fminf(sm1, fmaxf(((px + 1.f) / 2.f) * sm1, 0.f));
    const float iy = fminf(sm1, fmaxf(((py + 1.f) / 2.f) * sm1, 0.f));
    const float iz = fminf(sm1, fmaxf(((pz + 1.f) / 2.f) * sm1, 0.f));
    const float x0 = floorf(ix), y0 = floorf(iy), z0 = floorf(iz);
    const float wx1 = ix - x0, wx0 = (x0 + 1.f) - ix;
    const float wy1 = iy - y0, wy0 = (y0 + 1.f) - iy;
    const float wz1 = iz - z0, wz0 = (z0 + 1.f) - iz;
    const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
    // vertex index < 513^3 < 2^28 for the volumes the model check admits
    packed = (uint32_t)((zi * s + yi) * s + xi) | ((uint32_t)(xi + 1 < s) << 28) | ((uint32_t)(yi + 1 < s) << 29) |
             ((uint32_t)(zi + 1 < s) << 30);
    const float wxy[4] = {wx0 * wy0, wx1 * wy0, wx0 * wy1, wx1 * wy1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        w[k] = wxy[k] * wz0;
        w[k + 4] = wxy[k] * wz1;
    }
}

// corner_set for a point whose clamped grid coordinates are already known
// (the same expressions, so the same bits): vertex index of corner 0, the
// x / y / z neighbour flags (whether they differ from it) and the weights.
__device__ __forceinline__ void corner_set_at(int s, float ix, float iy, float iz, int &v0, bool &nx, bool &ny,
                                              bool &nz, float (&w)[8]) {
    const float x0 = floorf(ix), y0 = floorf(iy), z0 = floorf(iz);
    const float wx1 = ix - x0, wx0 = (x0 + 1.f) - ix;
    const float wy1 = iy - y0, wy0 = (y0 + 1.f) - iy;
    const float wz1 = iz - z0, wz0 = (z0 + 1.f) - iz;
    const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
    v0 = (zi * s + yi) * s + xi;
    nx = xi + 1 < s;
    ny = yi + 1 < s;
    nz = zi + 1 < s;
    const float wxy[4] = {wx0 * wy0, wx1 * wy0, wx0 * wy1, wx1 * wy1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        w[k] = wxy[k] * wz0;
        w[k + 4] = wxy[k] * wz1;
    }
}

// Sum over LODs 0..L of the trilinear samples of the 32 points of a warp
// (lane i owns point i's position).  Each lane computes its own point's
// corner set once per LOD; the loads are then done by LPP lanes per point
// (each owning 32/LPP channels, one 16-byte load per 8 channels and corner),
// which fetch the corner set from the point's lane with shuffles.  Pass p
// covers points p*(32/LPP) .. +32/LPP-1; acc[p] are this lane's channels
// (part = lane % LPP) of point p*(32/LPP) + lane / LPP, in fp32: per LOD the
// eight weighted corners are summed in order from zero with packed FMAs and
// the sample is added to the running sum.
template <int LPP>
__device__ __forceinline__ void gather_warp_rows(const nglod_bf16_model &m, int L, float px, float py, float pz,
                                                 int lane, float2 (&acc)[LPP][16 / LPP]) {
    constexpr int kQ = 16 / LPP;  // float2 per lane per point
    constexpr int kU = kQ / 4;    // 16-byte loads per corner
    const unsigned FULL = 0xffffffffu;
    const int part = lane % LPP;
#pragma unroll
    for (int p = 0; p < LPP; ++p)
#pragma unroll
        for (int c = 0; c < kQ; ++c) acc[p][c] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int l = m.summed ? L : 0; l <= L; ++l) {
        const uint4 *g = static_cast<const uint4 *>(m.grid[l]);  // 4 uint4 per vertex
        const int s = (1 << (l + m.base_lod)) + 1;
        const int sy = s * 4, sz = s * sy;
        uint32_t pk;
        float w[8];
        corner_set(s, px, py, pz, pk, w);
#pragma unroll
        for (int p = 0; p < LPP; ++p) {
            const int src = p * (32 / LPP) + lane / LPP;
            const uint32_t q = __shfl_sync(FULL, pk, src);
            float ws[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) ws[k] = __shfl_sync(FULL, w[k], src);
            const int o0 = (int)(q & 0x0FFFFFFFu) * 4 + part * kU;
            const int ox = ((q >> 28) & 1u) ? 4 : 0;
            const int oy = ((q >> 29) & 1u) ? sy : 0;
            const int oz = ((q >> 30) & 1u) ? sz : 0;
            const int o[8] = {o0, o0 + ox, o0 + oy, o0 + oy + ox, o0 + oz, o0 + oz + ox, o0 + oz + oy, o0 + oz + oy + ox};
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                uint4 v[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) v[k] = __ldg(g + o[k] + u);
                float2 a2[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                                make_float2(0.f, 0.f)};
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const float2 w2 = make_float2(ws[k], ws[k]);
                    a2[0] = __ffma2_rn(make_float2(bf_lo(v[k].x), bf_hi(v[k].x)), w2, a2[0]);
                    a2[1] = __ffma2_rn(make_float2(bf_lo(v[k].y), bf_hi(v[k].y)), w2, a2[1]);
                    a2[2] = __ffma2_rn(make_float2(bf_lo(v[k].z), bf_hi(v[k].z)), w2, a2[2]);
                    a2[3] = __ffma2_rn(make_float2(bf_lo(v[k].w), bf_hi(v[k].w)), w2, a2[3]);
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[p][4 * u + c] = __fadd2_rn(acc[p][4 * u + c], a2[c]);
            }
        }
    }
}

// Pair lines: vertex (z, y, x) of a volume stored beside its +x neighbour
// (x + 1 clamped to s - 1) as one 128-byte line of four 32-byte units, unit c
// = [v(z, y, x) channels 8c..8c+7 | v(z, y, x+1) channels 8c..8c+7]
// (PairUnit, ld_pair_unit: bf16_tile.cuh).

// gather_warp_rows<4> over pair volumes for the warp's 8 * NP points (lane
// i and every lane i + 8 * NP hold point i's position): the four lanes of a
// point (4j .. 4j + 3) each read one 32-byte unit of each of the point's
// four (y, z) lines, so a load instruction covers eight whole 128-byte lines
// (the vertex layout covers eight half lines) and each quarter warp two.
// (Lane i reading unit i / 8 of point i % 8 instead spreads a quarter warp
// over eight lines and made the kernel twice as slow.)  Each lane holds both x corners of its 8
// channels, and the eight weighted corners are summed in the same order
// (tnw..bse) as gather_warp_rows, so the two give identical sums.
template <int NP, typename Load>
__device__ __forceinline__ void pairs_add_level(int s, float px, float py, float pz, int lane, float2 (&acc)[NP][4],
                                                Load load) {
    const unsigned FULL = 0xffffffffu;
    const int sy = s * 4, sz = s * sy;
    // each lane's own point's clamped grid coordinates; the loading lanes
    // receive them by three shuffles and derive the corner set themselves
    // (corner_set's expressions: the same sums as shuffling its results)
    const float sm1 = (float)(s - 1);
    const float ix = fminf(sm1, fmaxf(((px + 1.f) / 2.f) * sm1, 0.f));
    const float iy = fminf(sm1, fmaxf(((py + 1.f) / 2.f) * sm1, 0.f));
    const float iz = fminf(sm1, fmaxf(((pz + 1.f) / 2.f) * sm1, 0.f));
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int src = p * 8 + (lane >> 2);
        const float qx = __shfl_sync(FULL, ix, src);
        const float qy = __shfl_sync(FULL, iy, src);
        const float qz = __shfl_sync(FULL, iz, src);
        float ws[8];
        int v0;
        bool nx, ny, nz;  // the pair line holds the x neighbour already
        corner_set_at(s, qx, qy, qz, v0, nx, ny, nz, ws);
        const int o0 = v0 * 4;
        const int oy = ny ? sy : 0;
        const int oz = nz ? sz : 0;
        const int o[4] = {o0, o0 + oy, o0 + oz, o0 + oz + oy};
        PairUnit v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = load(o[j]);
        float2 a2[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const float2 w2 = make_float2(ws[2 * j + x], ws[2 * j + x]);
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    a2[c] = __ffma2_rn(make_float2(bf_lo(v[j].w[4 * x + c]), bf_hi(v[j].w[4 * x + c])), w2, a2[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[p][c] = __fadd2_rn(acc[p][c], a2[c]);
    }
}

template <int NP>
__device__ __forceinline__ void gather_warp_pairs(const nglod_bf16_model &m, int L, float px, float py, float pz,
                                                  int lane, float2 (&acc)[NP][4]) {
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[p][c] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int l = m.summed ? L : 0; l <= L; ++l) {
        const PairUnit *g = static_cast<const PairUnit *>(m.grid_pairs[l]) + (lane & 3);  // 4 units per line
        pairs_add_level<NP>((1 << (l + m.base_lod)) + 1, px, py, pz, lane, acc,
                            [g](int o) { return ld_pair_unit(g + o); });
    }
}

// pairs_add_level's sums over a vertex volume (four 16-byte pieces per
// vertex; load(o) returns piece o of this lane's part): the eight corners are
// separate loads, summed in the same order (tnw..bse) with the same weights,
// so the results are identical.  Used for the volumes staged in shared
// memory, where the 64-byte vertices need no selects to spread a load
// instruction over the banks.
template <int NP, typename Load>
__device__ __forceinline__ void verts_add_level(int s, float px, float py, float pz, int lane, float2 (&acc)[NP][4],
                                                Load load) {
    const unsigned FULL = 0xffffffffu;
    const int sy = s * 4, sz = s * sy;
    const float sm1 = (float)(s - 1);
    const float ix = fminf(sm1, fmaxf(((px + 1.f) / 2.f) * sm1, 0.f));
    const float iy = fminf(sm1, fmaxf(((py + 1.f) / 2.f) * sm1, 0.f));
    const float iz = fminf(sm1, fmaxf(((pz + 1.f) / 2.f) * sm1, 0.f));
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int src = p * 8 + (lane >> 2);
        const float qx = __shfl_sync(FULL, ix, src);
        const float qy = __shfl_sync(FULL, iy, src);
        const float qz = __shfl_sync(FULL, iz, src);
        float ws[8];
        int v0;
        bool nx, ny, nz;
        corner_set_at(s, qx, qy, qz, v0, nx, ny, nz, ws);
        const int o0 = v0 * 4;
        const int ox = nx ? 4 : 0;
        const int oy = ny ? sy : 0;
        const int oz = nz ? sz : 0;
        const int o[8] = {o0, o0 + ox, o0 + oy, o0 + oy + ox, o0 + oz, o0 + oz + ox, o0 + oz + oy, o0 + oz + oy + ox};
        uint4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = load(o[k]);
        float2 a2[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float2 w2 = make_float2(ws[k], ws[k]);
            a2[0] = __ffma2_rn(make_float2(bf_lo(v[k].x), bf_hi(v[k].x)), w2, a2[0]);
            a2[1] = __ffma2_rn(make_float2(bf_lo(v[k].y), bf_hi(v[k].y)), w2, a2[1]);
            a2[2] = __ffma2_rn(make_float2(bf_lo(v[k].z), bf_hi(v[k].z)), w2, a2[2]);
            a2[3] = __ffma2_rn(make_float2(bf_lo(v[k].w), bf_hi(v[k].w)), w2, a2[3]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[p][c] = __fadd2_rn(acc[p][c], a2[c]);
    }
}

// Writes the tile rows row0 .. row0 + 8 * NP - 1 of gather_warp_pairs<NP>:
// every lane its 8 bf16 features of each pass's point, and lane i < 8 * NP
// the position / bias columns 32..39 of row row0 + i.
template <int NP>
__device__ __forceinline__ void write_pair_rows(uint8_t *sA, int row0, int lane, const float2 (&acc)[NP][4], float px,
                                                float py, float pz) {
    const int part = lane & 3;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int row = row0 + p * 8 + (lane >> 2);
        const uint4 f = make_uint4(pack_bf16x2(acc[p][0].x, acc[p][0].y), pack_bf16x2(acc[p][1].x, acc[p][1].y),
                                   pack_bf16x2(acc[p][2].x, acc[p][2].y), pack_bf16x2(acc[p][3].x, acc[p][3].y));
        *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, 8 * part)) = f;
    }
    if (lane < 8 * NP)
        *reinterpret_cast<uint4 *>(sA + tile_offset_a(row0 + lane, 32)) = position_columns(px, py, pz);
}

// Pair volume of a bf16 volume (s vertices per side), in 16-byte units:
// unit 8v + 2c + h of the pair volume is unit 4v' + c of the volume, v' = v
// for h = 0 and the +x neighbour (clamped) for h = 1.
__global__ void build_pairs_kernel(const uint4 *__restrict__ grid, int s, int64_t units, uint4 *__restrict__ pairs) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < units; i += stride) {
        const int64_t v = i >> 3;
        const int c = (int)((i >> 1) & 3), h = (int)(i & 1);
        const int64_t src = v + ((h && (v % s) + 1 < s) ? 1 : 0);
        pairs[i] = grid[4 * src + c];
    }
}

// LOD-summed volume L: vertex (z, y, x) of LOD L's grid holds the sum over
// LODs i <= L of volume i's trilinear sample at that vertex.  Grid spacings
// halve from LOD to LOD, so the vertex lies at coarse coordinate
// (x >> (L - i)) + fraction (x mod 2^(L-i)) / 2^(L-i) of volume i, and every
// cell of LOD L lies inside one cell of each coarser grid: a trilinear
// function restricted to a sub-box is trilinear, so trilinear sampling of
// this volume equals the sum of the per-LOD samples (with the same border
// clamp) up to rounding.  Samples and sum in float64 (dyadic weights, exact
// products), one rounding to T (float or bf16).  Thread per (vertex, channel).
template <typename T>
__global__ void build_summed_kernel(const nglod_dense_model m, int L, int64_t count, T *__restrict__ out) {
    const int C = m.feature_dim;
    const int sL = (1 << (L + m.base_lod)) + 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += stride) {
        const int c = (int)(t % C);
        const int64_t v = t / C;
        const int ix = (int)(v % sL), iy = (int)((v / sL) % sL), iz = (int)(v / ((int64_t)sL * sL));
        double sum = 0.0;
        for (int i = 0; i <= L; ++i) {
            const int sh = L - i, s = (1 << (i + m.base_lod)) + 1;
            const double inv = 1.0 / (double)(1 << sh);
            const int x0 = ix >> sh, y0 = iy >> sh, z0 = iz >> sh;
            const double fx = (ix & ((1 << sh) - 1)) * inv, fy = (iy & ((1 << sh) - 1)) * inv,
                         fz = (iz & ((1 << sh) - 1)) * inv;
            const int x1 = min(x0 + 1, s - 1), y1 = min(y0 + 1, s - 1), z1 = min(z0 + 1, s - 1);
            const float *g = static_cast<const float *>(m.grid[i]);
            auto at = [&](int z, int y, int x) { return (double)g[(((int64_t)z * s + y) * s + x) * C + c]; };
            const double c00 = at(z0, y0, x0) * (1.0 - fx) + at(z0, y0, x1) * fx;
            const double c01 = at(z0, y1, x0) * (1.0 - fx) + at(z0, y1, x1) * fx;
            const double c10 = at(z1, y0, x0) * (1.0 - fx) + at(z1, y0, x1) * fx;
            const double c11 = at(z1, y1, x0) * (1.0 - fx) + at(z1, y1, x1) * fx;
            sum += (c00 * (1.0 - fy) + c01 * fy) * (1.0 - fz) + (c10 * (1.0 - fy) + c11 * fy) * fz;
        }
        if constexpr (sizeof(T) == 4)
            out[t] = (float)sum;
        else
            out[t] = __double2bfloat16(sum);
    }
}

// Writes the warp's 32 tile rows (32w .. 32w+31): every lane its 32/LPP bf16
// features of each pass's point, and lane i the position / bias columns
// 32..39 of row 32w + i.
template <int LPP>
__device__ __forceinline__ void write_warp_rows(uint8_t *sA, int warp, int lane, const float2 (&acc)[LPP][16 / LPP],
                                                float px, float py, float pz) {
    constexpr int kQ = 16 / LPP;
    const int part = lane % LPP;
#pragma unroll
    for (int p = 0; p < LPP; ++p) {
        const int row = warp * 32 + p * (32 / LPP) + lane / LPP;
#pragma unroll
        for (int j = 0; j < kQ / 4; ++j) {
            const uint4 f = make_uint4(pack_bf16x2(acc[p][4 * j].x, acc[p][4 * j].y),
                                       pack_bf16x2(acc[p][4 * j + 1].x, acc[p][4 * j + 1].y),
                                       pack_bf16x2(acc[p][4 * j + 2].x, acc[p][4 * j + 2].y),
                                       pack_bf16x2(acc[p][4 * j + 3].x, acc[p][4 * j + 3].y));
            *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, 2 * kQ * part + 8 * j)) = f;
        }
    }
    *reinterpret_cast<uint4 *>(sA + tile_offset_a(warp * 32 + lane, 32)) = position_columns(px, py, pz);
}

// The tracer's gather: two lanes per point, each computing the corner set
// itself (neighbouring rays keep the lines of a load instruction shared; the
// tracer's own ray state leaves no registers for the warp-wide corner sets).
// Adds this lane's 16 channels (16h .. 16h+15) of the trilinear sample of
// one bf16 volume (s vertices per side) at p to acc; PyTorch grid_sample
// arithmetic (align_corners, border clamp), corners in tnw..bse order.  Two
// lanes share a point: each loads 2 x 16 bytes per corner, and the corner
// index / weight math is done once per 16 channels.
__device__ __forceinline__ void gather_bf16_half(const __nv_bfloat16 *__restrict__ g, int s, float px, float py,
                                                 float pz, int h, float (&acc)[16]) {
    const float sm1 = (float)(s - 1);
    const float ix = fminf(sm1, fmaxf(((px + 1.f) / 2.f) * sm1, 0.f));
    const float iy = fminf(sm1, fmaxf(((py + 1.f) / 2.f) * sm1, 0.f));
    const float iz = fminf(sm1, fmaxf(((pz + 1.f) / 2.f) * sm1, 0.f));
    const float x0 = floorf(ix), y0 = floorf(iy), z0 = floorf(iz);
    const float wx1 = ix - x0, wx0 = (x0 + 1.f) - ix;
    const float wy1 = iy - y0, wy0 = (y0 + 1.f) - iy;
    const float wz1 = iz - z0, wz0 = (z0 + 1.f) - iz;
    const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
    const int xj = min(xi + 1, s - 1), yj = min(yi + 1, s - 1), zj = min(zi + 1, s - 1);
    const uint4 *base = reinterpret_cast<const uint4 *>(g) + 2 * h;  // 4 uint4 per vertex
    // uint4 offsets fit in 32 bits (volumes up to 513^3 x 64 B)
    const int sy = s * 4, sz = s * sy;
    const int o0 = zi * sz + yi * sy + xi * 4;
    const int ox = (xj - xi) * 4, oy = (yj - yi) * sy, oz = (zj - zi) * sz;
    const int o[8] = {o0, o0 + ox, o0 + oy, o0 + oy + ox, o0 + oz, o0 + oz + ox, o0 + oz + oy, o0 + oz + oy + ox};
    const float wxy[4] = {wx0 * wy0, wx1 * wy0, wx0 * wy1, wx1 * wy1};
    const float w[8] = {wxy[0] * wz0, wxy[1] * wz0, wxy[2] * wz0, wxy[3] * wz0,
                        wxy[0] * wz1, wxy[1] * wz1, wxy[2] * wz1, wxy[3] * wz1};
    uint4 v[8], u[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = __ldg(base + o[k]);
        u[k] = __ldg(base + o[k] + 1);
    }
    // Packed fp32 FMAs (two channels per instruction) on the unpacked bf16 pairs.
    float2 a2[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) a2[c] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float2 w2 = make_float2(w[k], w[k]);
        a2[0] = __ffma2_rn(make_float2(bf_lo(v[k].x), bf_hi(v[k].x)), w2, a2[0]);
        a2[1] = __ffma2_rn(make_float2(bf_lo(v[k].y), bf_hi(v[k].y)), w2, a2[1]);
        a2[2] = __ffma2_rn(make_float2(bf_lo(v[k].z), bf_hi(v[k].z)), w2, a2[2]);
        a2[3] = __ffma2_rn(make_float2(bf_lo(v[k].w), bf_hi(v[k].w)), w2, a2[3]);
        a2[4] = __ffma2_rn(make_float2(bf_lo(u[k].x), bf_hi(u[k].x)), w2, a2[4]);
        a2[5] = __ffma2_rn(make_float2(bf_lo(u[k].y), bf_hi(u[k].y)), w2, a2[5]);
        a2[6] = __ffma2_rn(make_float2(bf_lo(u[k].z), bf_hi(u[k].z)), w2, a2[6]);
        a2[7] = __ffma2_rn(make_float2(bf_lo(u[k].w), bf_hi(u[k].w)), w2, a2[7]);
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        acc[2 * c] += a2[c].x;
        acc[2 * c + 1] += a2[c].y;
    }
}

// Writes a point's tile row from one of its two lanes: this lane's 16
// summed features (bf16, K columns 16h .. 16h+15) and, from h == 0, the
// position / bias columns 32..39.
__device__ __forceinline__ void write_tile_row_half(uint8_t *sA, int row, int h, const float (&acc)[16], float px,
                                                    float py, float pz) {
    constexpr int kCh = 16;
#pragma unroll
    for (int j = 0; j < kCh / 8; ++j) {
        const uint4 f = make_uint4(pack_bf16x2(acc[8 * j], acc[8 * j + 1]), pack_bf16x2(acc[8 * j + 2], acc[8 * j + 3]),
                                   pack_bf16x2(acc[8 * j + 4], acc[8 * j + 5]),
                                   pack_bf16x2(acc[8 * j + 6], acc[8 * j + 7]));
        *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, kCh * h + 8 * j)) = f;
    }
    if (h == 0) *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, 32)) = position_columns(px, py, pz);
}

// Ray entry into [-1,1]^3 with sol_nglod_kernel.cu:92-150's float arithmetic
// (same as the float32 path's box_entry).
__device__ __forceinline__ bool box_entry_bf(float ox, float oy, float oz, float dx, float dy, float dz, float &t) {
    const float ivx = (float)(1.0 / (double)dx);
    const float ivy = (float)(1.0 / (double)dy);
    const float ivz = (float)(1.0 / (double)dz);
    const float s0 = signbit(dx) ? 1.f : -1.f;
    const float s1 = signbit(dy) ? 1.f : -1.f;
    const float s2 = signbit(dz) ? 1.f : -1.f;
    const float cmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
    if (cmax < 1.f) return false;
    const float d0 = __fmul_rn(__fsub_rn(s0, ox), ivx);
    const float d1 = __fmul_rn(__fsub_rn(s1, oy), ivy);
    const float d2 = __fmul_rn(__fsub_rn(s2, oz), ivz);
    const bool t0 = (d0 >= 0.f) && (fabsf(fmaf(dy, d0, oy)) < 1.f) && (fabsf(fmaf(dz, d0, oz)) < 1.f);
    const bool t1 = (d1 >= 0.f) && (fabsf(fmaf(dx, d1, ox)) < 1.f) && (fabsf(fmaf(dz, d1, oz)) < 1.f);
    const bool t2 = (d2 >= 0.f) && (fabsf(fmaf(dx, d2, ox)) < 1.f) && (fabsf(fmaf(dy, d2, oy)) < 1.f);
    const float dd = t0 ? d0 : (t1 ? d1 : (t2 ? d2 : 0.f));
    if ((t0 || t1 || t2) && dd < 500.f) {
        t = dd;
        return true;
    }
    return false;
}

struct Bf16Args {
    nglod_bf16_model m;
    const float *x;
    int64_t n;
    int L;
    float *out;
    int *status;
    uint32_t wait_polls;  // bound of the per-tile tensor-core wait (nglod_debug_mma_wait_polls)
};

// Bound of the per-tile tensor-core wait of nglod_sdf_fwd_bf16 (host side,
// all devices): kWaitPolls unless a test of the error path lowers it.
static uint32_t g_bf16_wait_polls = kWaitPolls;

// One 128-point tile per block of four warps (models without pair
// volumes): warp w gathers rows 32w .. 32w + 31 from the vertex volumes, one
// thread issues the MMA, and thread (w, lane) runs the epilogue of TMEM lane
// / row 32w + lane.
__global__ void __launch_bounds__(kTP, 4) sdf_fwd_bf16_tc_kernel(const Bf16Args a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem + kSmemA;
    uint8_t *sB = smem + kSmemB;
    float *sb0 = reinterpret_cast<float *>(smem + kSmemB0);
    float *sw1 = reinterpret_cast<float *>(smem + kSmemW1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kSmemBar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSmemSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kSmemAbort);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint4 *bsrc = static_cast<const uint4 *>(a.m.w0_tile[a.L]);
    for (int i = tid; i < (int)(kTileBytes / 16); i += kTP) reinterpret_cast<uint4 *>(sB)[i] = bsrc[i];
    sb0[tid] = a.m.b0[a.L][tid];
    sw1[tid] = a.m.w1[a.L][tid];
    const float b1 = a.m.b1[a.L][0];
    // K core-matrix column 5 (k 40..47) is always zero.
    for (int i = tid; i < (kTP / 8) * 8; i += kTP) {
        const int grp = i >> 3, r = i & 7;
        *reinterpret_cast<uint4 *>(sA + grp * kSboA + 5 * kLboA + r * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (warp == 0) tc::tmem_alloc(slot, kHid);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        *abort_flag = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t sa = tc::smem_addr(sA), sb = tc::smem_addr(sB);
    const uint32_t idesc = tc::idesc_bf16_f32(kTP, kHid);
    uint32_t phase = 0;
    // unsorted query points: four lanes per point load (one load instruction
    // covers a point's 64-byte vertex)
    constexpr int kLPP = 4;

    for (int64_t tile = blockIdx.x; tile * kTP < a.n; tile += gridDim.x) {
        // 1. gather: warp w fills rows 32w .. 32w+31; lane i owns point 32w + i
        {
            const int64_t gi = tile * kTP + warp * 32 + lane;
            float px = 0.f, py = 0.f, pz = 0.f;
            if (gi < a.n) {
                px = a.x[3 * gi];
                py = a.x[3 * gi + 1];
                pz = a.x[3 * gi + 2];
            }
            float2 acc[kLPP][16 / kLPP];
            gather_warp_rows<kLPP>(a.m, a.L, px, py, pz, lane, acc);
            write_warp_rows<kLPP>(sA, warp, lane, acc, px, py, pz);
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        // 2. one thread issues the three K steps and commits to the barrier
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int ks = 0; ks < kTK / 16; ++ks) {
                const uint64_t ad = tc::smem_desc(sa + ks * 2 * kLboA, kLboA, kSboA);
                const uint64_t bd = tc::smem_desc(sb + ks * 256, kLbo, kSbo);
                tc::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
            tc::mma_commit(bar);
            if (!tc::mbar_wait_bounded(bar, phase, a.wait_polls)) {
                *abort_flag = 1;
                atomicExch(a.status, 1);
            }
        }
        __syncthreads();
        if (*abort_flag) break;
        phase ^= 1u;
        tc::fence_after_sync();
        // 3. epilogue: thread (w, lane) owns TMEM lane / tile row 32w + lane
        {
            float o = relu_dot_w1(tmem + ((uint32_t)(warp * 32) << 16), sw1);
            const int64_t gi = tile * kTP + warp * 32 + lane;
            if (gi < a.n) a.out[gi] = o + b1;
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (*abort_flag && tid == 0) tc::mbar_wait_bounded(bar, phase, kWaitPolls);  // let an in-flight MMA finish
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kHid);
}


// ---------------------------------------------------------------------------
// point query over pair volumes: persistent, coarse volumes in shared memory
// ---------------------------------------------------------------------------
// One 16-warp block per SM.  The leading volumes that fit (5^3 and 9^3
// vertices, 55 KB as bf16 vertex volumes, at base_lod 2) are copied into
// shared memory once per block and gathered corner by corner
// (verts_add_level); the finer levels come through L2 as pair lines with
// 32-byte loads.  The block is
// four independent groups of four warps, each with its own point tile and
// its own 128 TMEM columns (4 x 128 = the SM's 512): a group gathers 128
// points, writes their rows, its first thread issues the three K steps and
// waits, and the group runs the epilogue while the other groups gather.
// Groups meet only at their own named barrier (id 1 + g, 128 threads).
// Same arithmetic as sdf_fwd_bf16_tc_kernel over vertex volumes (identical
// results).
namespace b16st {
constexpr int kGroups = 4;
constexpr int kThreads = kTP * kGroups;  // 512
constexpr size_t kA = 0;                 // group g's point tile at kA + g kTileBytesA
constexpr size_t kB = kA + (size_t)kGroups * kTileBytesA;
constexpr size_t kW1 = kB + kTileBytes;
constexpr size_t kBar = kW1 + kHid * 4;  // one mbarrier per group
constexpr size_t kOk = kBar + 8 * kGroups;
constexpr size_t kSlot = kOk + 4 * kGroups;
constexpr size_t kAbort = kSlot + 4;
constexpr size_t kVol = (kAbort + 4 + 127) & ~(size_t)127;
constexpr size_t kSmemMax = 227 * 1024;
constexpr size_t kVolBudget = kSmemMax - kVol;
// more than half of an SM's shared memory: one block (512 TMEM columns) per SM
constexpr size_t kSmemMin = 120 * 1024;
constexpr uint32_t kCols = kGroups * kHid;
static_assert(kB % 16 == 0 && kBar % 8 == 0 && kVol % 128 == 0, "shared layout alignment");
static_assert(kVol + 54656 <= kSmemMax, "levels 5^3 and 9^3 fit");
}  // namespace b16st

__device__ __forceinline__ void b16_group_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "n"(kTP) : "memory");
}

// Levels first .. first + nstaged - 1 are staged (in that order) in shared
// memory; first = L for LOD-summed models, else 0.
__global__ void __launch_bounds__(b16st::kThreads, 1)
    sdf_fwd_bf16_staged_kernel(const Bf16Args a, int first, int nstaged) {
    using namespace b16st;
    extern __shared__ __align__(1024) uint8_t smem_b16st[];
    uint8_t *sm = smem_b16st;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = warp >> 2, quad = warp & 3, gtid = tid & (kTP - 1);
    uint8_t *sA = sm + kA + (size_t)grp * kTileBytesA;
    const float *sw1 = reinterpret_cast<const float *>(sm + kW1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBar) + grp;
    volatile int *okf = reinterpret_cast<volatile int *>(sm + kOk) + grp;
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + kSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    const int L = a.L;

    // set-up: decoder tile, w1, the zero K columns 40..47 of the point
    // tiles, the staged pair volumes, TMEM, barriers
    const uint4 *bsrc = static_cast<const uint4 *>(a.m.w0_tile[L]);
    for (int i = tid; i < (int)(kTileBytes / 16); i += kThreads) reinterpret_cast<uint4 *>(sm + kB)[i] = bsrc[i];
    if (tid < kHid) reinterpret_cast<float *>(sm + kW1)[tid] = a.m.w1[L][tid];
    const float b1 = a.m.b1[L][0];
    for (int i = tid; i < kGroups * (kTP / 8) * 8; i += kThreads) {
        const int g = i / ((kTP / 8) * 8), r8 = (i >> 3) % (kTP / 8), r = i & 7;
        *reinterpret_cast<uint4 *>(sm + kA + (size_t)g * kTileBytesA + r8 * kSboA + 5 * kLboA + r * 16) =
            make_uint4(0u, 0u, 0u, 0u);
    }
    {
        size_t off = kVol;
        for (int l = first; l < first + nstaged; ++l) {
            const int s = (1 << (l + a.m.base_lod)) + 1;
            const int cnt = s * s * s * 4;  // 16-byte pieces
            const uint4 *src = static_cast<const uint4 *>(a.m.grid[l]);
            uint4 *dst = reinterpret_cast<uint4 *>(sm + off);
            for (int q = tid; q < cnt; q += kThreads) dst[q] = src[q];
            off += (size_t)cnt * 16;
        }
    }
    if (warp == 0) tc::tmem_alloc(slot, kCols);
    if (tid == 0) {
        for (int g = 0; g < kGroups; ++g) tc::mbar_init(reinterpret_cast<uint64_t *>(sm + kBar) + g, 1);
        *abort_flag = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t dcol = tmem + (uint32_t)(grp * kHid);
    const uint32_t sa = tc::smem_addr(sA), sb = tc::smem_addr(sm + kB);
    const uint32_t idesc = tc::idesc_bf16_f32(kTP, kHid);
    const int part = lane & 3;
    uint32_t phase = 0;
    bool pending = false;  // group leader: an issued product whose completion it did not see

    const int64_t stride = (int64_t)gridDim.x * kGroups;
    // this thread's point of the group's next tile, loaded one tile ahead (the
    // points may be host memory read over the host link)
    float nx = 0.f, ny = 0.f, nz = 0.f;
    {
        const int64_t i0 = ((int64_t)blockIdx.x * kGroups + grp) * kTP + gtid;
        if (i0 < a.n) {
            nx = a.x[3 * i0];
            ny = a.x[3 * i0 + 1];
            nz = a.x[3 * i0 + 2];
        }
    }
    for (int64_t t = (int64_t)blockIdx.x * kGroups + grp; t * kTP < a.n; t += stride) {
        const int64_t gi = t * kTP + gtid;
        const float px = nx, py = ny, pz = nz;
        {
            const int64_t in = gi + stride * kTP;
            nx = ny = nz = 0.f;
            if (in < a.n) {
                nx = a.x[3 * in];
                ny = a.x[3 * in + 1];
                nz = a.x[3 * in + 2];
            }
        }
        // 1. gather: the warp's 32 points (rows 32 quad ..), staged levels
        // from shared memory, the rest from the pair volumes in global memory
        float2 acc[4][4];
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[p][c] = make_float2(0.f, 0.f);
        const uint4 *vol = reinterpret_cast<const uint4 *>(sm + kVol) + part;  // 4 pieces per vertex
#pragma unroll 1
        for (int l = first; l < first + nstaged; ++l) {
            const int s = (1 << (l + a.m.base_lod)) + 1;
            verts_add_level<4>(s, px, py, pz, lane, acc, [vol](int o) { return vol[o]; });
            vol += s * s * s * 4;
        }
#pragma unroll 1
        for (int l = first + nstaged; l <= L; ++l) {
            const PairUnit *g = static_cast<const PairUnit *>(a.m.grid_pairs[l]) + part;
            pairs_add_level<4>((1 << (l + a.m.base_lod)) + 1, px, py, pz, lane, acc,
                               [g](int o) { return ld_pair_unit(g + o); });
        }
        write_pair_rows<4>(sA, quad * 32, lane, acc, px, py, pz);
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        b16_group_sync(grp);
        // 2. the group's first thread issues the three K steps and waits (not
        // once another group's wait gave up: the group then stops)
        if (gtid == 0) {
            bool ok = false;
            if (!*abort_flag) {
                tc::fence_after_sync();
#pragma unroll
                for (int ks = 0; ks < kTK / 16; ++ks) {
                    const uint64_t ad = tc::smem_desc(sa + ks * 2 * kLboA, kLboA, kSboA);
                    const uint64_t bd = tc::smem_desc(sb + ks * 256, kLbo, kSbo);
                    tc::mma_bf16(dcol, ad, bd, idesc, ks > 0 ? 1u : 0u);
                }
                tc::mma_commit(bar);
                ok = tc::mbar_wait_bounded(bar, phase, a.wait_polls);
                if (!ok) {
                    pending = true;
                    *abort_flag = 1;
                    atomicExch(a.status, 1);
                }
            }
            *okf = ok ? 1 : 0;
        }
        b16_group_sync(grp);
        if (!*okf) break;
        phase ^= 1u;
        tc::fence_after_sync();
        // 3. epilogue on this thread's TMEM row
        const float o = relu_dot_w1(dcol + ((uint32_t)(quad * 32) << 16), sw1);
        if (gi < a.n) a.out[gi] = o + b1;
        tc::fence_before_sync();
    }
    // teardown: a product still in flight after a wait gave up finishes
    // before the columns are freed
    if (gtid == 0 && pending) tc::mbar_wait_bounded(bar, phase, kWaitPolls);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------------------
// persistent BF16 sphere tracer
// ---------------------------------------------------------------------------
// 128 ray slots per block, one per thread.  Every iteration each slot
// publishes one query point (the ray's next march point or one of its six
// normal taps), the block gathers and decodes all 128 points as one tile
// (above), and each thread advances its ray with SphereTracer.forward's state
// machine (sdf-net/lib/tracer/SphereTracer.py:74-130, same rules as the float32
// persistent tracer).  Finished slots write their ray out and take the next
// ray index from a global counter, one atomicAdd per warp.
struct Bf16TraceArgs {
    nglod_bf16_model m;
    nglod_trace_params p;
    int L;
    const float *ray_o;
    const float *ray_d;
    int64_t n;
    float *x;
    float *t;
    uint8_t *hit;
    float *normal;
    unsigned long long *counter;
    int *status;
};

enum : int { bNeed = 0, bEvalInit = 1, bMarch = 2, bTap0 = 3, bDone = 9, bGone = 10 };

__global__ void __launch_bounds__(kTP, 4) trace_bf16_tc_kernel(const Bf16TraceArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem + kSmemA;
    uint8_t *sB = smem + kSmemB;
    float *sb0 = reinterpret_cast<float *>(smem + kSmemB0);
    float *sw1 = reinterpret_cast<float *>(smem + kSmemW1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kSmemBar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSmemSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kSmemAbort);
    float4 *qpts = reinterpret_cast<float4 *>(smem + kSmemQ);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint4 *bsrc = static_cast<const uint4 *>(a.m.w0_tile[a.L]);
    for (int i = tid; i < (int)(kTileBytes / 16); i += kTP) reinterpret_cast<uint4 *>(sB)[i] = bsrc[i];
    sb0[tid] = a.m.b0[a.L][tid];
    sw1[tid] = a.m.w1[a.L][tid];
    const float b1 = a.m.b1[a.L][0];
    for (int i = tid; i < (kTP / 8) * 8; i += kTP) {
        const int grp = i >> 3, r = i & 7;
        *reinterpret_cast<uint4 *>(sA + grp * kSboA + 5 * kLboA + r * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (warp == 0) tc::tmem_alloc(slot, kHid);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        *abort_flag = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t sa = tc::smem_addr(sA), sb = tc::smem_addr(sB);
    const uint32_t idesc = tc::idesc_bf16_f32(kTP, kHid);
    uint32_t mphase = 0;
    // neighbouring rays query nearby points: two lanes per point (the cache
    // lines of a load instruction are shared by neighbouring points)
    constexpr int kLPP = 2;

    const unsigned FULL = 0xffffffffu;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float h = 1.0f / 192.0f;
    const float twoh = (float)(2.0 / 192.0);
    int phase = bNeed, step = 0;
    int64_t ray = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f;
    // t is carried as an unevaluated sum t + tc: each step adds d with
    // Knuth's TwoSum and keeps the rounding error in tc (compensated
    // summation), so 64+ steps of small d do not drift; te = t + tc is the
    // depth used for positions, the far-clip test and the output.
    float xx = 0.f, xy = 0.f, xz = 0.f, t = 0.f, tc = 0.f, te = 0.f, d = 0.f, dprev = 0.f;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nx = 0.f, ny = 0.f, nz = 0.f;
    bool cond = false, hitr = false, hitf = false;

    auto finish = [&]() {
        hitf = hitr && !(fabsf(xx) > 1.f || fabsf(xy) > 1.f || fabsf(xz) > 1.f);
        phase = (hitf && a.p.want_normals) ? bTap0 : bDone;
    };
    auto march_decide = [&]() {
        if (step >= a.p.num_steps) {
            finish();
            return;
        }
        hitr = fabsf(te) < a.p.far_clip;
        cond = cond && (fabsf(d) > a.p.min_dis) && (fabsf((d + dprev) / 2.f) > a.p.osc_dis) && hitr;
        if (!cond) {
            finish();
            return;
        }
        xx = __fadd_rn(ox, __fmul_rn(dx, te));
        xy = __fadd_rn(oy, __fmul_rn(dy, te));
        xz = __fadd_rn(oz, __fmul_rn(dz, te));
        dprev = d;
        phase = bMarch;
    };

    for (;;) {
        for (;;) {
            if (phase == bDone) {
                a.x[3 * ray + 0] = xx;
                a.x[3 * ray + 1] = xy;
                a.x[3 * ray + 2] = xz;
                a.t[ray] = te;
                a.hit[ray] = hitf ? 1 : 0;
                if (a.normal) {
                    const bool hn = hitf && a.p.want_normals;
                    a.normal[3 * ray + 0] = hn ? nx : 0.f;
                    a.normal[3 * ray + 1] = hn ? ny : 0.f;
                    a.normal[3 * ray + 2] = hn ? nz : 0.f;
                }
                phase = bNeed;
            }
            const unsigned need = __ballot_sync(FULL, phase == bNeed);
            if (need == 0u) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0ull;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (phase == bNeed) {
                const unsigned long long r = base + (unsigned long long)__popc(need & lt_mask);
                if (r >= (unsigned long long)a.n) {
                    phase = bGone;
                } else {
                    ray = (int64_t)r;
                    ox = a.ray_o[3 * ray];
                    oy = a.ray_o[3 * ray + 1];
                    oz = a.ray_o[3 * ray + 2];
                    dx = a.ray_d[3 * ray];
                    dy = a.ray_d[3 * ray + 1];
                    dz = a.ray_d[3 * ray + 2];
                    t = 0.f;
                    cond = box_entry_bf(ox, oy, oz, dx, dy, dz, t);
                    tc = 0.f;
                    te = t;
                    xx = cond ? fmaf(dx, t, ox) : ox;
                    xy = cond ? fmaf(dy, t, oy) : oy;
                    xz = cond ? fmaf(dz, t, oz) : oz;
                    step = 0;
                    hitr = false;
                    hitf = false;
                    if (cond)
                        phase = bEvalInit;
                    else
                        march_decide();
                }
            }
        }
        if (__syncthreads_and(phase == bGone)) break;

        float qx = xx, qy = xy, qz = xz;
        if (phase >= bTap0 && phase < bDone) {
            const int k = phase - bTap0;
            const float e = (k & 1) ? -h : h;
            if ((k >> 1) == 0) qx = __fadd_rn(xx, e);
            else if ((k >> 1) == 1) qy = __fadd_rn(xy, e);
            else qz = __fadd_rn(xz, e);
        }
        if (phase == bGone) qx = qy = qz = 0.f;
        qpts[tid] = make_float4(qx, qy, qz, 0.f);
        __syncthreads();
#pragma unroll 1
        for (int pass = 0; pass < kLPP; ++pass) {
            const int row = warp * 32 + pass * (32 / kLPP) + lane / kLPP;
            const float4 pt = qpts[row];
            float acc[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) acc[c] = 0.f;
#pragma unroll 1
            for (int l = a.m.summed ? a.L : 0; l <= a.L; ++l)
                gather_bf16_half(static_cast<const __nv_bfloat16 *>(a.m.grid[l]), (1 << (l + a.m.base_lod)) + 1, pt.x,
                                 pt.y, pt.z, lane % kLPP, acc);
            write_tile_row_half(sA, row, lane % kLPP, acc, pt.x, pt.y, pt.z);
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int ks = 0; ks < kTK / 16; ++ks) {
                const uint64_t ad = tc::smem_desc(sa + ks * 2 * kLboA, kLboA, kSboA);
                const uint64_t bd = tc::smem_desc(sb + ks * 256, kLbo, kSbo);
                tc::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
            tc::mma_commit(bar);
            if (!tc::mbar_wait_bounded(bar, mphase, kWaitPolls)) {
                *abort_flag = 1;
                atomicExch(a.status, 1);
            }
        }
        __syncthreads();
        if (*abort_flag) break;
        mphase ^= 1u;
        tc::fence_after_sync();
        float v = relu_dot_w1(tmem + ((uint32_t)(warp * 32) << 16), sw1) + b1;
        tc::fence_before_sync();

        if (phase == bEvalInit) {
            d = v;
            dprev = d;
            march_decide();
        } else if (phase == bMarch) {
            d = v * a.p.step_size;
            const float tsum = __fadd_rn(t, d);
            const float bp = __fsub_rn(tsum, t);
            const float err = __fadd_rn(__fsub_rn(t, __fsub_rn(tsum, bp)), __fsub_rn(d, bp));
            t = tsum;
            tc = __fadd_rn(tc, err);
            te = __fadd_rn(t, tc);
            ++step;
            march_decide();
        } else if (phase >= bTap0 && phase < bDone) {
            const int k = phase - bTap0;
#pragma unroll
            for (int i = 0; i < 6; ++i)
                if (i == k) g[i] = v;
            if (k == 5) {
                const float gx = (g[0] - g[1]) / twoh;
                const float gy = (g[2] - g[3]) / twoh;
                const float gz = (g[4] - g[5]) / twoh;
                const float nrm = sqrtf(gx * gx + gy * gy + gz * gz);
                const float den = fmaxf(nrm, 1e-5f);
                nx = gx / den;
                ny = gy / den;
                nz = gz / den;
                phase = bDone;
            } else {
                phase = phase + 1;
            }
        }
    }
    if (*abort_flag && tid == 0) tc::mbar_wait_bounded(bar, mphase, kWaitPolls);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kHid);
}

}  // namespace nglod

using namespace nglod;

extern "C" int nglod_bf16_pack_decoder(const float *w0_host, const float *b0_host, int32_t hidden_dim, int32_t in_dim,
                                       void *tile_host) {
    NGLOD_REQUIRE(w0_host && b0_host && tile_host, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(hidden_dim == kHid && in_dim == 35, NGLOD_ERR_UNSUPPORTED,
                  "bf16 decoder tile built for w0 [128][35], got [%d][%d]", hidden_dim, in_dim);
    uint16_t *t = static_cast<uint16_t *>(tile_host);
    memset(t, 0, kTileBytes);
    for (int n = 0; n < kHid; ++n) {
        for (int k = 0; k < kTK; ++k) {
            float w = 0.f;
            if (k < 32) w = w0_host[n * 35 + 3 + k];
            else if (k < 35) w = w0_host[n * 35 + (k - 32)];
            else if (k < 38) w = w0_host[n * 35 + (k - 35)];
            else if (k == 38) w = __bfloat162float(__float2bfloat16_rn(b0_host[n]));
            else if (k == 39) w = b0_host[n] - __bfloat162float(__float2bfloat16_rn(b0_host[n]));
            const __nv_bfloat16 b = __float2bfloat16_rn(w);
            uint16_t bits;
            memcpy(&bits, &b, 2);
            t[tc::tile_offset(n, k, kKC) / 2] = bits;
        }
    }
    return NGLOD_OK;
}

// zero_status: reset *status on the stream first (the public call); the
// host-memory pipeline resets it once for all of its chunks.
static int sdf_fwd_bf16_impl(const nglod_bf16_model *model, const float *x, int64_t n, int32_t lod, float *out,
                             int32_t *status, cudaStream_t s, bool zero_status) {
    NGLOD_REQUIRE(model != nullptr, NGLOD_ERR_INVALID, "model is null");
    NGLOD_REQUIRE(model->num_lods >= 1 && model->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID, "num_lods=%d",
                  model->num_lods);
    NGLOD_REQUIRE(model->feature_dim == 32 && model->hidden_dim == kHid, NGLOD_ERR_UNSUPPORTED,
                  "bf16 form built for feature_dim 32 and hidden_dim 128");
    NGLOD_REQUIRE(model->base_lod >= 0 && model->num_lods - 1 + model->base_lod <= 9, NGLOD_ERR_INVALID,
                  "base_lod=%d", model->base_lod);
    const int L = (lod < 0 || lod >= model->num_lods) ? model->num_lods - 1 : lod;
    for (int l = 0; l <= L; ++l)
        NGLOD_REQUIRE(model->grid[l] && aligned(model->grid[l], 16), NGLOD_ERR_ALIGN,
                      "bf16 volume %d is null or not 16-byte aligned", l);
    NGLOD_REQUIRE(model->w0_tile[L] && aligned(model->w0_tile[L], 16) && model->b0[L] && model->w1[L] &&
                      model->b1[L],
                  NGLOD_ERR_INVALID, "decoder %d: null or misaligned tile/bias pointer", L);
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && out && status, NGLOD_ERR_INVALID, "null pointer argument");
    bool pairs = true;
    for (int l = 0; l <= L; ++l) {
        NGLOD_REQUIRE(!model->grid_pairs[l] || aligned(model->grid_pairs[l], 32), NGLOD_ERR_ALIGN,
                      "bf16 pair volume %d is not 32-byte aligned", l);
        pairs = pairs && model->grid_pairs[l] != nullptr;
    }
    if (zero_status)
        NGLOD_TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int32_t), s), "nglod_sdf_fwd_bf16 memset"));
    Bf16Args a;
    a.m = *model;
    a.x = x;
    a.n = n;
    a.L = L;
    a.out = out;
    a.status = status;
    a.wait_polls = g_bf16_wait_polls;
    const int64_t tiles = (n + kTP - 1) / kTP;
    if (pairs) {
        // the leading pair volumes that fit beside the tiles are staged
        const int first = model->summed ? L : 0;
        int nstaged = 0;
        size_t vbytes = 0;
        for (int l = first; l <= L; ++l) {
            const size_t sd = (size_t)(1 << (l + model->base_lod)) + 1;
            if (vbytes + sd * sd * sd * 64 > b16st::kVolBudget) break;
            vbytes += sd * sd * sd * 64;
            ++nstaged;
        }
        const size_t smem = b16st::kVol + vbytes < b16st::kSmemMin ? b16st::kSmemMin : b16st::kVol + vbytes;
        NGLOD_TRY(cuda_status(cudaFuncSetAttribute(sdf_fwd_bf16_staged_kernel,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                              "cudaFuncSetAttribute"));
        const int64_t want = (tiles + b16st::kGroups - 1) / b16st::kGroups;
        const int64_t cap = (int64_t)num_sms();
        sdf_fwd_bf16_staged_kernel<<<(int)(want < cap ? want : cap), b16st::kThreads, smem, s>>>(a, first, nstaged);
        return launch_status("nglod_sdf_fwd_bf16");
    }
    NGLOD_TRY(cuda_status(cudaFuncSetAttribute(sdf_fwd_bf16_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kSmemBytes),
                          "cudaFuncSetAttribute"));
    const int64_t cap = (int64_t)num_sms() * 4;
    sdf_fwd_bf16_tc_kernel<<<(int)(tiles < cap ? tiles : cap), kTP, kSmemBytes, s>>>(a);
    return launch_status("nglod_sdf_fwd_bf16");
}

extern "C" int nglod_bf16_build_pairs(const void *grid, int32_t s, void *pairs, nglod_stream_t stream) {
    NGLOD_REQUIRE(grid && pairs, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(s >= 2 && s <= 1025, NGLOD_ERR_INVALID, "s=%d", s);
    NGLOD_REQUIRE(aligned(grid, 16) && aligned(pairs, 32), NGLOD_ERR_ALIGN,
                  "grid must be 16-byte and pairs 32-byte aligned");
    const int64_t units = (int64_t)s * s * s * 8;
    const int64_t want = (units + 255) / 256, cap = (int64_t)num_sms() * 16;
    build_pairs_kernel<<<(int)(want < cap ? want : cap), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const uint4 *>(grid), s, units, static_cast<uint4 *>(pairs));
    return launch_status("nglod_bf16_build_pairs");
}

extern "C" int nglod_build_summed_volume(const nglod_dense_model *model, int32_t lod, int32_t dtype, void *out,
                                         nglod_stream_t stream) {
    NGLOD_REQUIRE(model && out, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(model->feature_dim == 32, NGLOD_ERR_INVALID, "feature_dim=%d (32 supported)", model->feature_dim);
    NGLOD_REQUIRE(model->base_lod >= 0 && model->num_lods - 1 + model->base_lod <= 9, NGLOD_ERR_INVALID,
                  "base_lod=%d num_lods=%d", model->base_lod, model->num_lods);
    NGLOD_REQUIRE(lod >= 0 && lod < model->num_lods, NGLOD_ERR_INVALID, "lod=%d outside 0..%d", lod,
                  model->num_lods - 1);
    NGLOD_REQUIRE(dtype == NGLOD_F32 || dtype == NGLOD_BF16, NGLOD_ERR_INVALID, "dtype=%d", dtype);
    for (int l = 0; l <= lod; ++l) NGLOD_REQUIRE(model->grid[l], NGLOD_ERR_INVALID, "volume %d is null", l);
    NGLOD_REQUIRE(aligned(out, 16), NGLOD_ERR_ALIGN, "out must be 16-byte aligned");
    const int64_t s = ((int64_t)1 << (lod + model->base_lod)) + 1;
    const int64_t count = s * s * s * 32;
    const int grid = (int)std::min<int64_t>((count + 255) / 256, (int64_t)num_sms() * 16);
    if (dtype == NGLOD_F32)
        build_summed_kernel<float><<<grid, 256, 0, (cudaStream_t)stream>>>(*model, lod, count, static_cast<float *>(out));
    else
        build_summed_kernel<__nv_bfloat16>
            <<<grid, 256, 0, (cudaStream_t)stream>>>(*model, lod, count, static_cast<__nv_bfloat16 *>(out));
    return launch_status("nglod_build_summed_volume");
}

// Read throughput of random whole 128-byte lines of a buffer, with the
// point-query gather's loads (four lanes per line, one 256-bit load each, a
// warp covering eight lines per instruction).  For a buffer the size of the
// pair volumes, held in L2, this is the measured ceiling of the gather's
// corner reads.  Line indices: xorshift32 per group of four lanes (never
// zero), taken modulo `lines`, so every load is in bounds.
__global__ void line_read_kernel(const PairUnit *__restrict__ buf, uint32_t lines, int loads, uint32_t seed,
                                 uint32_t *__restrict__ sink) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t h = ((t >> 2) * 2654435761u) ^ seed;
    h |= 1u;
    uint32_t acc = 0u;
    const PairUnit *base = buf + (threadIdx.x & 3);
#pragma unroll 4
    for (int k = 0; k < loads; ++k) {
        h ^= h << 13;
        h ^= h >> 17;
        h ^= h << 5;
        const PairUnit u = ld_pair_unit(base + (size_t)(h % lines) * 4);
        acc ^= u.w[0] ^ u.w[1] ^ u.w[2] ^ u.w[3] ^ u.w[4] ^ u.w[5] ^ u.w[6] ^ u.w[7];
    }
    if (acc == 0x9E3779B9u) sink[0] = t;  // keeps every load
}

extern "C" int nglod_measure_line_reads(const void *buf, int64_t lines, int32_t loads, int32_t blocks,
                                        uint32_t *sink, nglod_stream_t stream) {
    NGLOD_REQUIRE(buf && sink, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(buf, 32), NGLOD_ERR_ALIGN, "buf must be 32-byte aligned");
    NGLOD_REQUIRE(lines >= 1 && lines <= 0xFFFFFFFFll, NGLOD_ERR_INVALID, "lines=%lld", (long long)lines);
    NGLOD_REQUIRE(loads >= 1 && blocks >= 1, NGLOD_ERR_INVALID, "loads=%d blocks=%d", loads, blocks);
    line_read_kernel<<<blocks, 128, 0, (cudaStream_t)stream>>>(static_cast<const PairUnit *>(buf), (uint32_t)lines,
                                                               loads, 0x2545F491u, sink);
    return launch_status("nglod_measure_line_reads");
}

extern "C" int nglod_sdf_fwd_bf16(const nglod_bf16_model *model, const float *x, int64_t n, int32_t lod, float *out,
                                  int32_t *status, nglod_stream_t stream) {
    return sdf_fwd_bf16_impl(model, x, n, lod, out, status, (cudaStream_t)stream, true);
}

namespace {
struct Bf16HostCtx {
    const nglod_bf16_model *model;
    int32_t lod;
    int32_t *status;
};
int bf16_host_chunk(const void *ctx, const float *x, int64_t m, float *out, cudaStream_t s) {
    const Bf16HostCtx *c = static_cast<const Bf16HostCtx *>(ctx);
    return sdf_fwd_bf16_impl(c->model, x, m, c->lod, out, c->status, s, false);
}
}  // namespace

extern "C" int nglod_sdf_fwd_bf16_host(const nglod_bf16_model *model, const float *x_host, int64_t n, int32_t lod,
                                       float *out_host, int64_t chunk, void *scratch, int32_t *status,
                                       nglod_stream_t stream) {
    NGLOD_TRY(sdf_fwd_bf16_impl(model, nullptr, 0, lod, nullptr, nullptr, nullptr, false));  // validates the model
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(status, NGLOD_ERR_INVALID, "null pointer argument");
    cudaStream_t s = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int32_t), s), "nglod_sdf_fwd_bf16_host memset"));
    const Bf16HostCtx ctx{model, lod, status};
    return host_query_pipeline(x_host, n, out_host, chunk, scratch, s, bf16_host_chunk, &ctx);
}

extern "C" int nglod_trace_bf16(const nglod_bf16_model *model, const nglod_trace_params *params, const float *ray_o,
                                const float *ray_d, int64_t n, float *x, float *t, uint8_t *hit, float *normal,
                                int64_t *work_counter, int32_t *status, nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr && params != nullptr, NGLOD_ERR_INVALID, "model or params is null");
    NGLOD_REQUIRE(model->num_lods >= 1 && model->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID, "num_lods=%d",
                  model->num_lods);
    NGLOD_REQUIRE(model->feature_dim == 32 && model->hidden_dim == kHid, NGLOD_ERR_UNSUPPORTED,
                  "bf16 form built for feature_dim 32 and hidden_dim 128");
    NGLOD_REQUIRE(model->base_lod >= 0 && model->num_lods - 1 + model->base_lod <= 9, NGLOD_ERR_INVALID,
                  "base_lod=%d", model->base_lod);
    NGLOD_REQUIRE(params->num_steps >= 0, NGLOD_ERR_INVALID, "num_steps=%d is negative", params->num_steps);
    const int L = (params->lod < 0 || params->lod >= model->num_lods) ? model->num_lods - 1 : params->lod;
    for (int l = 0; l <= L; ++l)
        NGLOD_REQUIRE(model->grid[l] && aligned(model->grid[l], 16), NGLOD_ERR_ALIGN,
                      "bf16 volume %d is null or not 16-byte aligned", l);
    NGLOD_REQUIRE(model->w0_tile[L] && aligned(model->w0_tile[L], 16) && model->b0[L] && model->w1[L] &&
                      model->b1[L],
                  NGLOD_ERR_INVALID, "decoder %d: null or misaligned tile/bias pointer", L);
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && x && t && hit && work_counter && status, NGLOD_ERR_INVALID,
                  "null pointer argument");
    NGLOD_REQUIRE(normal || !params->want_normals, NGLOD_ERR_INVALID, "normals requested with a null buffer");
    NGLOD_REQUIRE(aligned(work_counter, 8), NGLOD_ERR_ALIGN, "work_counter is not 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int32_t), s), "nglod_trace_bf16 memset"));
    NGLOD_TRY(cuda_status(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), s), "nglod_trace_bf16 memset"));
    Bf16TraceArgs a;
    a.m = *model;
    a.p = *params;
    a.L = L;
    a.ray_o = ray_o;
    a.ray_d = ray_d;
    a.n = n;
    a.x = x;
    a.t = t;
    a.hit = hit;
    a.normal = normal;
    a.counter = reinterpret_cast<unsigned long long *>(work_counter);
    a.status = status;
    NGLOD_TRY(cuda_status(
        cudaFuncSetAttribute(trace_bf16_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes),
        "cudaFuncSetAttribute"));
    const int64_t want = (n + kTP - 1) / kTP;
    const int64_t cap = (int64_t)num_sms() * 4;
    trace_bf16_tc_kernel<<<(int)(want < cap ? want : cap), kTP, kSmemBytes, s>>>(a);
    return launch_status("nglod_trace_bf16");
}

extern "C" int nglod_debug_mma_wait_polls(int64_t polls) {
    NGLOD_REQUIRE(polls <= (int64_t)kWaitPolls, NGLOD_ERR_INVALID, "polls=%lld above the default %u",
                  (long long)polls, kWaitPolls);
    g_bf16_wait_polls = polls < 0 ? kWaitPolls : (uint32_t)polls;
    set_f32tc_wait_polls(g_bf16_wait_polls);
    return NGLOD_OK;
}
