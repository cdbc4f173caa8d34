// Device building blocks of the dense float32 path shared by the forward,
// tracer and training kernels.
//
// Layout: feature volume l is channel-last [s][s][s][C] (C = 32 floats =
// 128 B per vertex), so each trilinear corner is one cache line, read by
// eight lanes with one 16-byte load each.  The decoder of one LOD is staged
// in shared memory as H rows of 36 floats (35 weights of Linear(35, H)
// followed by its bias; the input vector carries a trailing 1.0) plus the H
// weights and the bias of Linear(H, 1).  Every thread decodes whole points,
// reading the decoder rows as warp-wide broadcasts.
#pragma once

#include <math.h>

#include "common.cuh"

namespace nglod {

constexpr int kC = 32;         // feature channels this library is built for
constexpr int kRowF4 = 9;      // float4 per staged decoder row (35 weights + bias)

// float4 count of one staged decoder with H hidden units.
__host__ __device__ inline int decoder_f4(int H) { return H * kRowF4 + (H + 4) / 4; }

// Stages decoder (w0 [H][35], b0 [H], w1 [H], b1 [1]) into dst as H rows of
// 36 floats (row weights then bias) followed by w1 and b1.
__device__ __forceinline__ void stage_decoder_ptrs(float4 *dst, int H, const float *__restrict__ w0,
                                                   const float *__restrict__ b0, const float *__restrict__ w1,
                                                   const float *__restrict__ b1) {
    float *rows = reinterpret_cast<float *>(dst);
    for (int i = threadIdx.x; i < H * 36; i += blockDim.x) {
        const int j = i / 36, k = i - j * 36;
        rows[i] = k < 35 ? w0[j * 35 + k] : b0[j];
    }
    float *w1s = rows + H * 36;
    for (int j = threadIdx.x; j < H; j += blockDim.x) w1s[j] = w1[j];
    if (threadIdx.x == 0) w1s[H] = b1[0];
}

__device__ __forceinline__ void stage_decoder(float4 *dst, const nglod_dense_model &m, int l) {
    stage_decoder_ptrs(dst, m.hidden_dim, m.w0[l], m.b0[l], m.w1[l], m.b1[l]);
}

// Adds the trilinear samples of one channel-last float32 volume (s vertices
// per side) at the warp's 32 points (lane i owns point i's position).  Same
// arithmetic as PyTorch's 3-D grid sampler with align_corners=True and
// padding_mode='border': u = ((p + 1) / 2) * (s - 1) clamped to [0, s - 1],
// corner weights are products of distances to the opposite corner, corners
// summed in tnw, tne, tsw, tse, bnw, bne, bsw, bse order from zero per
// channel, then added to the running sum.  The far corner index is clamped
// to s - 1 where u = s - 1; its weight is then exactly 0, as when PyTorch
// skips the out-of-range corner.
// Cooperative loads: in pass p the eight lanes 8j .. 8j + 7 load the
// corners of point 4p + j, one float4 (channels 4 (lane % 8) .. +3) each, so
// a load instruction reads four whole 128-byte vertices instead of 16 bytes
// of 32 different ones.  Each lane computes its own point's clamped grid
// coordinates; the loading lanes receive them by three shuffles and derive
// the corner offsets and weights themselves (shuffling the corner index and
// the eight weights instead takes nine shuffles, which load the shared-memory
// crossbar the tensor-core kernels also use).  acc[p] += this lane's four
// channels of point 4p + lane / 8.
__device__ __forceinline__ void gather_warp_add_f32(const float *__restrict__ g, int s, float px, float py, float pz,
                                                    int lane, float4 (&acc)[8]) {
    const unsigned FULL = 0xffffffffu;
    const float sm1 = (float)(s - 1);
    float ix = ((px + 1.f) / 2.f) * sm1;
    float iy = ((py + 1.f) / 2.f) * sm1;
    float iz = ((pz + 1.f) / 2.f) * sm1;
    ix = fminf(sm1, fmaxf(ix, 0.f));
    iy = fminf(sm1, fmaxf(iy, 0.f));
    iz = fminf(sm1, fmaxf(iz, 0.f));
    const float4 *g4 = reinterpret_cast<const float4 *>(g) + (lane & 7);  // 8 float4 per vertex
    const int sy = s * 8, sz = s * sy;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const int src = 4 * p + (lane >> 3);
        const float qx = __shfl_sync(FULL, ix, src);
        const float qy = __shfl_sync(FULL, iy, src);
        const float qz = __shfl_sync(FULL, iz, src);
        const float x0 = floorf(qx), y0 = floorf(qy), z0 = floorf(qz);
        const float wx1 = qx - x0, wx0 = (x0 + 1.f) - qx;
        const float wy1 = qy - y0, wy0 = (y0 + 1.f) - qy;
        const float wz1 = qz - z0, wz0 = (z0 + 1.f) - qz;
        const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
        float ws[8];
        ws[0] = wx0 * wy0 * wz0;
        ws[1] = wx1 * wy0 * wz0;
        ws[2] = wx0 * wy1 * wz0;
        ws[3] = wx1 * wy1 * wz0;
        ws[4] = wx0 * wy0 * wz1;
        ws[5] = wx1 * wy0 * wz1;
        ws[6] = wx0 * wy1 * wz1;
        ws[7] = wx1 * wy1 * wz1;
        // vertex index < 513^3 < 2^28, float4 offsets < 2^31
        const int o0 = ((zi * s + yi) * s + xi) * 8;
        const int ox = xi + 1 < s ? 8 : 0;
        const int oy = yi + 1 < s ? sy : 0;
        const int oz = zi + 1 < s ? sz : 0;
        const int o[8] = {o0, o0 + ox, o0 + oy, o0 + oy + ox, o0 + oz, o0 + oz + ox, o0 + oz + oy, o0 + oz + oy + ox};
        float4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = __ldg(g4 + o[k]);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            a0 = fmaf(v[k].x, ws[k], a0);
            a1 = fmaf(v[k].y, ws[k], a1);
            a2 = fmaf(v[k].z, ws[k], a2);
            a3 = fmaf(v[k].w, ws[k], a3);
        }
        acc[p].x += a0;
        acc[p].y += a1;
        acc[p].z += a2;
        acc[p].w += a3;
    }
}

// gather_warp_add_f32 over a volume staged in shared memory (v points into
// the kernel's shared-memory array; channel-last, 128 B per vertex): the same
// expressions in the same order, so the same sums.
__device__ __forceinline__ void gather_warp_add_f32_shared(const float4 *v, int s, float px, float py, float pz,
                                                           int lane, float4 (&acc)[8]) {
    const unsigned FULL = 0xffffffffu;
    const float sm1 = (float)(s - 1);
    float ix = ((px + 1.f) / 2.f) * sm1;
    float iy = ((py + 1.f) / 2.f) * sm1;
    float iz = ((pz + 1.f) / 2.f) * sm1;
    ix = fminf(sm1, fmaxf(ix, 0.f));
    iy = fminf(sm1, fmaxf(iy, 0.f));
    iz = fminf(sm1, fmaxf(iz, 0.f));
    const float4 *g4 = v + (lane & 7);  // 8 float4 per vertex
    const int sy = s * 8, sz = s * sy;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const int src = 4 * p + (lane >> 3);
        const float qx = __shfl_sync(FULL, ix, src);
        const float qy = __shfl_sync(FULL, iy, src);
        const float qz = __shfl_sync(FULL, iz, src);
        const float x0 = floorf(qx), y0 = floorf(qy), z0 = floorf(qz);
        const float wx1 = qx - x0, wx0 = (x0 + 1.f) - qx;
        const float wy1 = qy - y0, wy0 = (y0 + 1.f) - qy;
        const float wz1 = qz - z0, wz0 = (z0 + 1.f) - qz;
        const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
        float ws[8];
        ws[0] = wx0 * wy0 * wz0;
        ws[1] = wx1 * wy0 * wz0;
        ws[2] = wx0 * wy1 * wz0;
        ws[3] = wx1 * wy1 * wz0;
        ws[4] = wx0 * wy0 * wz1;
        ws[5] = wx1 * wy0 * wz1;
        ws[6] = wx0 * wy1 * wz1;
        ws[7] = wx1 * wy1 * wz1;
        const int o0 = ((zi * s + yi) * s + xi) * 8;
        const int ox = xi + 1 < s ? 8 : 0;
        const int oy = yi + 1 < s ? sy : 0;
        const int oz = zi + 1 < s ? sz : 0;
        const int o[8] = {o0, o0 + ox, o0 + oy, o0 + oy + ox, o0 + oz, o0 + oz + ox, o0 + oz + oy, o0 + oz + oy + ox};
        float4 vv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) vv[k] = g4[o[k]];
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            a0 = fmaf(vv[k].x, ws[k], a0);
            a1 = fmaf(vv[k].y, ws[k], a1);
            a2 = fmaf(vv[k].z, ws[k], a2);
            a3 = fmaf(vv[k].w, ws[k], a3);
        }
        acc[p].x += a0;
        acc[p].y += a1;
        acc[p].z += a2;
        acc[p].w += a3;
    }
}

// Row stride (floats) of the per-warp transpose buffer: 36, so that the
// float4 reads of eight consecutive rows fall in different banks.
constexpr int kTRow = 36;

// Hands the cooperative sums back to the point owners through the warp's
// shared buffer sT [32][kTRow]: f = the 32 channels of point `lane`.
__device__ __forceinline__ void warp_sums_to_points(float *sT, int lane, const float4 (&acc)[8], float (&f)[kC]) {
#pragma unroll
    for (int p = 0; p < 8; ++p)
        *reinterpret_cast<float4 *>(sT + (4 * p + (lane >> 3)) * kTRow + 4 * (lane & 7)) = acc[p];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kC / 4; ++q) {
        const float4 v = *reinterpret_cast<const float4 *>(sT + lane * kTRow + 4 * q);
        f[4 * q] = v.x;
        f[4 * q + 1] = v.y;
        f[4 * q + 2] = v.z;
        f[4 * q + 3] = v.w;
    }
    __syncwarp();
}

// Linear(35, H) -> ReLU -> Linear(H, 1) on [p, f] with the staged decoder.
// kMask: also store the ReLU mask (bit j of word j / 32 = hidden unit j was
// positive) to mask_out[0 .. (H + 31) / 32 - 1] (nothing when mask_out is
// null).
template <bool kMask = false>
__device__ __forceinline__ float decode_f32(const float4 *__restrict__ dec, int H, float px, float py,
                                            float pz, const float (&f)[kC], uint32_t *mask_out = nullptr) {
    const float *__restrict__ w1 = reinterpret_cast<const float *>(dec + H * kRowF4);
    float in[36];
    in[0] = px;
    in[1] = py;
    in[2] = pz;
#pragma unroll
    for (int c = 0; c < kC; ++c) in[3 + c] = f[c];
    in[35] = 1.f;
    float out = 0.f;
    uint32_t bits = 0u;
#pragma unroll 1
    for (int j = 0; j < H; j += 2) {
        const float4 *r0 = dec + j * kRowF4;
        const float4 *r1 = r0 + kRowF4;
        float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
#pragma unroll
        for (int q = 0; q < kRowF4; ++q) {
            const float4 u = r0[q];
            const float4 v = r1[q];
            if (q & 1) {
                a1 = fmaf(u.x, in[4 * q + 0], a1);
                a1 = fmaf(u.y, in[4 * q + 1], a1);
                a1 = fmaf(u.z, in[4 * q + 2], a1);
                a1 = fmaf(u.w, in[4 * q + 3], a1);
                b1 = fmaf(v.x, in[4 * q + 0], b1);
                b1 = fmaf(v.y, in[4 * q + 1], b1);
                b1 = fmaf(v.z, in[4 * q + 2], b1);
                b1 = fmaf(v.w, in[4 * q + 3], b1);
            } else {
                a0 = fmaf(u.x, in[4 * q + 0], a0);
                a0 = fmaf(u.y, in[4 * q + 1], a0);
                a0 = fmaf(u.z, in[4 * q + 2], a0);
                a0 = fmaf(u.w, in[4 * q + 3], a0);
                b0 = fmaf(v.x, in[4 * q + 0], b0);
                b0 = fmaf(v.y, in[4 * q + 1], b0);
                b0 = fmaf(v.z, in[4 * q + 2], b0);
                b0 = fmaf(v.w, in[4 * q + 3], b0);
            }
        }
        const float h0 = fmaxf(a0 + a1, 0.f);
        const float h1 = fmaxf(b0 + b1, 0.f);
        out = fmaf(w1[j], h0, out);
        out = fmaf(w1[j + 1], h1, out);
        if (kMask) {
            bits |= ((uint32_t)(h0 > 0.f) << (j & 31)) | ((uint32_t)(h1 > 0.f) << ((j + 1) & 31));
            if (((j + 2) & 31) == 0 || j + 2 >= H) {
                if (mask_out) mask_out[j >> 5] = bits;
                bits = 0u;
            }
        }
    }
    return out + w1[H];
}

__device__ __forceinline__ int volume_side(const nglod_dense_model &m, int l) { return (1 << (l + m.base_lod)) + 1; }


// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
inline int check_model(const nglod_dense_model *m, int L_max) {
    NGLOD_REQUIRE(m != nullptr, NGLOD_ERR_INVALID, "model is null");
    NGLOD_REQUIRE(m->num_lods >= 1 && m->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID,
                  "num_lods=%d outside [1, %d]", m->num_lods, NGLOD_MAX_LODS);
    NGLOD_REQUIRE(m->base_lod >= 0 && m->num_lods - 1 + m->base_lod <= 9, NGLOD_ERR_INVALID,
                  "base_lod=%d with num_lods=%d gives volumes above 2^9+1 per side", m->base_lod, m->num_lods);
    NGLOD_REQUIRE(m->feature_dim == kC, NGLOD_ERR_UNSUPPORTED, "feature_dim=%d not built (only %d)",
                  m->feature_dim, kC);
    NGLOD_REQUIRE(m->hidden_dim >= 2 && m->hidden_dim <= 256 && (m->hidden_dim % 2) == 0, NGLOD_ERR_UNSUPPORTED,
                  "hidden_dim=%d not built (even, 2..256)", m->hidden_dim);
    NGLOD_REQUIRE(m->grid_dtype == NGLOD_F32, NGLOD_ERR_UNSUPPORTED, "grid_dtype=%d: this entry point is float32",
                  m->grid_dtype);
    for (int l = 0; l <= L_max; ++l) {
        NGLOD_REQUIRE(m->grid[l] && m->w0[l] && m->b0[l] && m->w1[l] && m->b1[l], NGLOD_ERR_INVALID,
                      "lod %d has a null volume or decoder pointer", l);
        NGLOD_REQUIRE(aligned(m->grid[l], 16), NGLOD_ERR_ALIGN, "volume %d is not 16-byte aligned", l);
    }
    return NGLOD_OK;
}

inline int resolve_lod(const nglod_dense_model *m, int lod) {
    return (lod < 0 || lod >= m->num_lods) ? m->num_lods - 1 : lod;
}

template <typename K>
inline int prepare_smem(K kernel, size_t smem) {
    NGLOD_REQUIRE(smem <= 227 * 1024, NGLOD_ERR_UNSUPPORTED, "decoder staging needs %zu B of shared memory", smem);
    return cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute");
}

template <typename K>
inline int resident_blocks(K kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * num_sms();
}

}  // namespace nglod
