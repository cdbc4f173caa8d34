// Training kernels of the dense float32 path: forward with saved feature
// sums and ReLU masks, hand-written backward, the L2 loss, multi-tensor Adam.
//
// Backward of one training batch (lod_mask = set of LODs with a loss term):
//   1. decoder part, per LOD l in the mask:
//      - hidden_dim 128 with the forward's ReLU masks:
//        sdf_bwd_decoder_tc_kernel, two tcgen05 products per 128-point tile
//        (dLoss/d(feature sum) and the weight-gradient accumulator), no
//        hidden layer recomputed;
//      - otherwise sdf_bwd_decoder_kernel: each point's hidden layer is
//        recomputed in float32 in the forward's order, dLoss/d(feature sum)
//        written, and the block reduces its tiles into the weight gradients.
//   2. sdf_bwd_scatter_kernel: per point, the gradient reaching volume i is
//      the suffix sum over mask LODs l >= i of dLoss/d(feature sum l); it is
//      scattered with the trilinear weights, eight lanes per point.  The
//      coarsest volumes (5^3 and 9^3 vertices at base_lod 2) are accumulated
//      in shared memory per block and flushed once; finer ones use
//      red.global.add.v4.f32.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "dense_common.cuh"
#include "tc_common.cuh"
#include "f32_tile.cuh"

namespace nglod {

constexpr int kBT = 128;  // points per backward tile = threads per block

__device__ int32_t g_train_status;  // nonzero: a tensor-core wait of a training kernel gave up

// ---------------------------------------------------------------------------
// forward for training
// ---------------------------------------------------------------------------
// Each warp evaluates 32 points at a time (lane i owns point base + i):
// cooperative LOD gathers (gather_warp_add_f32); after each LOD in the mask
// the running sums are written to feats straight from the cooperative layout
// (four whole rows per store instruction), handed to the point owners
// through the warp's shared buffer, and decoded by each lane.
constexpr int kFwdTrainThreads = 512;  // 16 warps share the staged decoders of all LODs

template <bool kRelu>
__global__ void __launch_bounds__(kFwdTrainThreads, 1)
    sdf_fwd_train_kernel(const nglod_dense_model m, const float *__restrict__ x, int64_t n, int L, uint32_t mask,
                         float *__restrict__ preds, float *__restrict__ feats, uint32_t *__restrict__ relu) {
    extern __shared__ float4 smem[];
    const int H = m.hidden_dim;
    const int dstride = decoder_f4(H);
    for (int l = 0; l <= L; ++l)
        if ((mask >> l) & 1u) stage_decoder(smem + l * dstride, m, l);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *sT = reinterpret_cast<float *>(smem + (L + 1) * dstride) + warp * 32 * kTRow;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + warp * 32; base < n; base += stride) {
        const int64_t i = base + lane;
        float px = 0.f, py = 0.f, pz = 0.f;
        if (i < n) {
            px = x[3 * i];
            py = x[3 * i + 1];
            pz = x[3 * i + 2];
        }
        float4 acc[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) acc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
        for (int l = 0; l <= L; ++l) {
            gather_warp_add_f32(static_cast<const float *>(m.grid[l]), volume_side(m, l), px, py, pz, lane, acc);
            if ((mask >> l) & 1u) {
#pragma unroll
                for (int p = 0; p < 8; ++p) {
                    const int64_t ip = base + 4 * p + (lane >> 3);
                    if (ip < n) reinterpret_cast<float4 *>(feats + ((int64_t)l * n + ip) * kC)[lane & 7] = acc[p];
                }
                float f[kC];
                warp_sums_to_points(sT, lane, acc, f);
                const int64_t row = (int64_t)l * n + i;
                const float o = decode_f32<kRelu>(smem + l * dstride, H, px, py, pz, f,
                                                  kRelu && i < n ? relu + row * ((H + 31) / 32) : nullptr);
                if (i < n) preds[row] = o;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// forward for training, tensor-core form (hidden_dim 128, ReLU masks wanted)
// ---------------------------------------------------------------------------
// The decoder's first layer, P [128 pts x 128 hid] = [F, x y z, 1] . [W, b0]^T,
// runs on tcgen05 as kind::tf32 products over big / small splits of both
// operands (the point tiles of f32_tile.cuh: relative error about 2^-21, the
// size of the float32 path's own rounding), accumulated in TMEM.  ReLU, the
// ReLU mask and the 128 -> 1 layer are a float32 epilogue per point.  Units
// whose pre-activation lies within the split products' error of zero (a few
// per thousand points) are evaluated again in float32 with the per-thread
// decoder's order, so that the saved ReLU mask is the float32 path's
// decision.
// A block of eight warps handles two 128-point tiles per iteration against
// one staged weight tile (the layout of the fused float32 tracer: warps 0-3
// fill tile 0, warps 4-7 tile 1; two blocks per SM hold 2 x 256 TMEM
// columns).  Blocks run LOD by LOD so that each LOD's weights are staged
// once: a block visits the same points at every LOD, and the running
// feature sum of a point is carried through feats (row l-1 is read back by
// the very lanes that wrote it), which therefore holds every row 0..L.
namespace fwdtc {
using f32tile::kH;
using f32tile::kK;
using f32tile::kTileA;
using f32tile::kTileF;
using f32tile::kTP;
using f32tile::kWBytes;
constexpr int kTiles = 2, kThreads = kTP * kTiles;
constexpr size_t kA = 0, kW = kTiles * kTileA, kW1 = kW + kWBytes;
constexpr size_t kBar = kW1 + kH * 4, kSlot = kBar + 8, kAbort = kSlot + 4;
constexpr size_t kSmem = kAbort + 12;
constexpr uint32_t kCols = kTiles * kH;
constexpr uint32_t kPolls = 1u << 22;
// |P| below which a unit's sign is settled by a float32 evaluation: above the
// split products' error (about 2^-21 of sum |w x|) for sums up to ~20
constexpr float kNearZero = 1e-5f;
static_assert(kW % 1024 == 0 && kBar % 8 == 0, "shared layout alignment");
static_assert(2 * (kSmem + 1024) <= 228 * 1024, "two blocks per SM");
}  // namespace fwdtc

// Hidden unit j's pre-activation for point row r of a point tile, in
// float32 with decode_f32's order (inputs x y z, features, 1; products of
// even and odd float4 groups summed apart, then added).  The features are
// big + small of the tile, which is exact.
__device__ __noinline__ float pre_f32(const uint8_t *tile, int r, float px, float py, float pz,
                                      const float *__restrict__ w0, const float *__restrict__ b0, int j) {
    using namespace fwdtc;
    auto in_at = [&](int k) -> float {  // decode_f32's input k
        if (k < 3) return k == 0 ? px : (k == 1 ? py : pz);
        if (k == 35) return 1.f;
        const uint32_t off = tile_offset32_sw128(r, k - 3);
        return *reinterpret_cast<const float *>(tile + off) + *reinterpret_cast<const float *>(tile + kTileF + off);
    };
    float a0 = 0.f, a1 = 0.f;
#pragma unroll 1
    for (int q = 0; q < 9; ++q) {
        float t = q & 1 ? a1 : a0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = 4 * q + e;
            t = fmaf(k < 35 ? w0[j * 35 + k] : b0[j], in_at(k), t);
        }
        if (q & 1)
            a1 = t;
        else
            a0 = t;
    }
    return a0 + a1;
}

__global__ void __launch_bounds__(fwdtc::kThreads, 2)
    sdf_fwd_train_tc_kernel(const nglod_dense_model m, const float *__restrict__ x, int64_t n, int L, uint32_t mask,
                            float *__restrict__ preds, float *__restrict__ feats, uint32_t *__restrict__ relu) {
    using namespace fwdtc;
    extern __shared__ __align__(1024) uint8_t smem_fw[];
    uint8_t *sm = smem_fw;
    const float *w1s = reinterpret_cast<const float *>(sm + kW1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + kSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int half = warp >> 2, quad = warp & 3;

    if (warp == 0) tc::tmem_alloc(slot, kCols);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        *abort_flag = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t sbase = tc::smem_addr(sm);
    uint8_t *tile = sm + kA + (size_t)half * kTileA;
    const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * kH);
    const int row = quad * 32 + lane;  // this thread's point row in its tile
    uint32_t phase = 0;

#pragma unroll 1
    for (int l = 0; l <= L && !*abort_flag; ++l) {
        const bool decode = (mask >> l) & 1u;
        // this LOD's decoder (the weight side of the point tiles, w1); the
        // previous LOD's products all completed before its last barrier
        if (decode) stage_tf32_decoder(m, l, sm + kW, sm + kW1, tid, kThreads);
        const float b1 = decode ? m.b1[l][0] : 0.f;
        const int s = volume_side(m, l);
#pragma unroll 1
        for (int64_t q = blockIdx.x; q * kThreads < n; q += gridDim.x) {
            const int64_t base = q * kThreads + warp * 32;
            const int64_t i = base + lane;
            float px = 0.f, py = 0.f, pz = 0.f;
            if (i < n) {
                px = x[3 * i];
                py = x[3 * i + 1];
                pz = x[3 * i + 2];
            }
            // running sum: LOD l's sample added to row l-1 of feats
            float4 acc[8];
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                const int64_t ip = base + 4 * p + (lane >> 3);
                acc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (l > 0 && ip < n)
                    acc[p] = reinterpret_cast<const float4 *>(feats + ((int64_t)(l - 1) * n + ip) * kC)[lane & 7];
            }
            gather_warp_add_f32(static_cast<const float *>(m.grid[l]), s, px, py, pz, lane, acc);
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                const int64_t ip = base + 4 * p + (lane >> 3);
                if (ip < n) reinterpret_cast<float4 *>(feats + ((int64_t)l * n + ip) * kC)[lane & 7] = acc[p];
            }
            if (!decode) continue;
            store_point_rows(tile, quad * 32, lane, acc, px, py, pz);
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
#pragma unroll
                for (int h = 0; h < kTiles; ++h)
                    issue_first_layer(tmem + (uint32_t)(h * kH), sbase + (uint32_t)(kA + h * kTileA),
                                      sbase + (uint32_t)kW);
                tc::mma_commit(bar);
                if (!tc::mbar_wait_bounded(bar, phase, kPolls)) {
                    *abort_flag = 1;
                    atomicExch(&g_train_status, 1);
                }
            }
            __syncthreads();
            if (*abort_flag) break;
            phase ^= 1u;
            tc::fence_after_sync();
            // epilogue: this thread's point (row quad * 32 + lane of tile half)
            float out = 0.f;
            uint32_t bits[4];
#pragma unroll 1
            for (int c = 0; c < 4; ++c) {
                float v[32];
                tc::tmem_load32(taddr + (uint32_t)(32 * c), v);
                uint32_t b = 0u, near = 0u;
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                    const float zv = v[e];
                    const bool z = fabsf(zv) < kNearZero;
                    near |= (uint32_t)z << e;
                    out = fmaf(w1s[32 * c + e], z ? 0.f : fmaxf(zv, 0.f), out);
                    b |= (uint32_t)(zv > 0.f && !z) << e;
                }
                while (near) {  // rare: a few units per thousand points
                    const int e = __ffs(near) - 1;
                    near &= near - 1u;
                    const float f = pre_f32(tile, row, px, py, pz, m.w0[l], m.b0[l], 32 * c + e);
                    if (f > 0.f) {
                        out = fmaf(w1s[32 * c + e], f, out);
                        b |= 1u << e;
                    }
                }
                bits[c] = b;
            }
            if (i < n) {
                const int64_t r = (int64_t)l * n + i;
                preds[r] = out + b1;
                reinterpret_cast<uint4 *>(relu)[r] = make_uint4(bits[0], bits[1], bits[2], bits[3]);
            }
            tc::fence_before_sync();
            __syncthreads();
        }
        __syncthreads();
    }
    if (*abort_flag && tid == 0) tc::mbar_wait_bounded(bar, phase, kPolls);  // let an in-flight product finish
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------------------
// backward 1: decoders
// ---------------------------------------------------------------------------
struct BwdArgs {
    nglod_dense_model m;
    nglod_dense_grads g;
    const float *x;
    int64_t n;
    uint32_t mask;
    int L;
    const float *gpred;
    const float *feats;
    const uint32_t *relu;  // forward ReLU masks [L+1][n][H/32] (tensor-core form)
    float *dfeat;
    float *gx;
};

// Backward tile: kBP points per tile, kBThreads threads per block.  Phase 1
// (per point): four threads per point, each recomputing a quarter of the
// hidden units (j = part, part+4, ...) and its share of dLoss/d(input); the
// four partial input gradients are summed with shuffles.  Phase 2 (per
// hidden unit): thread (j, half) reduces half of the tile's points into
// dW0[j][:], db0[j], dw1[j]; the two halves are added in turn.
constexpr int kBP = 64;
constexpr int kBThreads = 256;
static_assert(kBThreads == 4 * kBP && kBThreads == 2 * kBT, "backward tile shape");

__host__ __device__ inline int bwd_ht_floats(int H) { return kBP * (H + 1); }
// Shared layout (floats): decoder | H tile [kBP][H+1] | IN tile [kBP][36] | g [kBP] | acc [H][37]
__host__ __device__ inline size_t bwd_decoder_smem(int H) {
    size_t f = (size_t)decoder_f4(H) * 4 + bwd_ht_floats(H);
    f = (f + 3) & ~(size_t)3;
    return (f + kBP * 36 + kBP + (size_t)H * 37) * sizeof(float);
}

__global__ void __launch_bounds__(kBThreads, 2) sdf_bwd_decoder_kernel(const BwdArgs a) {
    extern __shared__ float4 smem[];
    const int H = a.m.hidden_dim;
    const int tid = threadIdx.x;
    float4 *dec = smem;
    float *Ht = reinterpret_cast<float *>(smem + decoder_f4(H));
    size_t off = (size_t)decoder_f4(H) * 4 + bwd_ht_floats(H);
    off = (off + 3) & ~(size_t)3;
    float *INt = reinterpret_cast<float *>(smem) + off;
    float *gt = INt + kBP * 36;
    float *acc = gt + kBP;
    const float *w1s = reinterpret_cast<const float *>(dec + H * kRowF4);
    const int pl = tid >> 2, part = tid & 3;      // phase 1: point of the tile, quarter
    const int jr = tid & (kBT - 1), half = tid / kBT;  // phase 2: hidden unit, half of the points

    for (int l = 0; l <= a.L; ++l) {
        if (!((a.mask >> l) & 1u)) continue;
        __syncthreads();
        stage_decoder(dec, a.m, l);
        for (int i = tid; i < H * 37; i += kBThreads) acc[i] = 0.f;
        float db1 = 0.f;
        __syncthreads();
        for (int64_t tile = blockIdx.x; tile * kBP < a.n; tile += gridDim.x) {
            const int64_t p = tile * kBP + pl;
            const bool valid = p < a.n;
            float in[36];
            float g = 0.f;
            if (valid) {
                in[0] = a.x[3 * p];
                in[1] = a.x[3 * p + 1];
                in[2] = a.x[3 * p + 2];
                const float4 *fr = reinterpret_cast<const float4 *>(a.feats + ((int64_t)l * a.n + p) * kC);
#pragma unroll
                for (int q = 0; q < kC / 4; ++q) {
                    const float4 v = fr[q];
                    in[3 + 4 * q] = v.x;
                    in[4 + 4 * q] = v.y;
                    in[5 + 4 * q] = v.z;
                    in[6 + 4 * q] = v.w;
                }
                in[35] = 1.f;
                g = a.gpred[(int64_t)l * a.n + p];
            } else {
#pragma unroll
                for (int k = 0; k < 36; ++k) in[k] = 0.f;
            }
            float din[36];
#pragma unroll
            for (int k = 0; k < 36; ++k) din[k] = 0.f;
#pragma unroll 1
            for (int j = part; j < H; j += 4) {
                const float4 *r = dec + j * kRowF4;
                float s0 = 0.f, s1 = 0.f;
#pragma unroll
                for (int q = 0; q < kRowF4; ++q) {
                    const float4 w = r[q];
                    if (q & 1) {
                        s1 = fmaf(w.x, in[4 * q], s1);
                        s1 = fmaf(w.y, in[4 * q + 1], s1);
                        s1 = fmaf(w.z, in[4 * q + 2], s1);
                        s1 = fmaf(w.w, in[4 * q + 3], s1);
                    } else {
                        s0 = fmaf(w.x, in[4 * q], s0);
                        s0 = fmaf(w.y, in[4 * q + 1], s0);
                        s0 = fmaf(w.z, in[4 * q + 2], s0);
                        s0 = fmaf(w.w, in[4 * q + 3], s0);
                    }
                }
                const float pre = s0 + s1;
                const float h = fmaxf(pre, 0.f);
                const float dh = pre > 0.f ? g * w1s[j] : 0.f;
                Ht[pl * (H + 1) + j] = h;
#pragma unroll
                for (int q = 0; q < kRowF4; ++q) {
                    const float4 w = r[q];
                    din[4 * q] = fmaf(dh, w.x, din[4 * q]);
                    din[4 * q + 1] = fmaf(dh, w.y, din[4 * q + 1]);
                    din[4 * q + 2] = fmaf(dh, w.z, din[4 * q + 2]);
                    din[4 * q + 3] = fmaf(dh, w.w, din[4 * q + 3]);
                }
            }
            // the point's four quarters are lanes 4i .. 4i+3 of one warp
#pragma unroll
            for (int k = 0; k < 35; ++k) {
                din[k] += __shfl_xor_sync(0xffffffffu, din[k], 1);
                din[k] += __shfl_xor_sync(0xffffffffu, din[k], 2);
            }
            if (valid) {
                float4 *o = reinterpret_cast<float4 *>(a.dfeat + ((int64_t)l * a.n + p) * kC);
#pragma unroll
                for (int q = 0; q < kC / 4; ++q)
                    if ((q >> 1) == part)
                        o[q] = make_float4(din[3 + 4 * q], din[4 + 4 * q], din[5 + 4 * q], din[6 + 4 * q]);
                if (a.gx && part == 0) {
                    a.gx[3 * p] += din[0];
                    a.gx[3 * p + 1] += din[1];
                    a.gx[3 * p + 2] += din[2];
                }
            }
            float4 *ir = reinterpret_cast<float4 *>(INt + pl * 36);
#pragma unroll
            for (int q = 0; q < 9; ++q)
                if ((q & 3) == part) ir[q] = make_float4(in[4 * q], in[4 * q + 1], in[4 * q + 2], in[4 * q + 3]);
            if (part == 0) gt[pl] = g;
            __syncthreads();
            float r[36];
#pragma unroll
            for (int k = 0; k < 36; ++k) r[k] = 0.f;
            float dw1 = 0.f;
            if (jr < H) {
                const float w1j = w1s[jr];
#pragma unroll 2
                for (int q = half * (kBP / 2); q < (half + 1) * (kBP / 2); ++q) {
                    const float h = Ht[q * (H + 1) + jr];
                    const float gq = gt[q];
                    const float dh = h > 0.f ? gq * w1j : 0.f;
                    dw1 = fmaf(gq, h, dw1);
                    const float4 *row = reinterpret_cast<const float4 *>(INt + q * 36);
#pragma unroll
                    for (int k4 = 0; k4 < 9; ++k4) {
                        const float4 v = row[k4];
                        r[4 * k4] = fmaf(dh, v.x, r[4 * k4]);
                        r[4 * k4 + 1] = fmaf(dh, v.y, r[4 * k4 + 1]);
                        r[4 * k4 + 2] = fmaf(dh, v.z, r[4 * k4 + 2]);
                        r[4 * k4 + 3] = fmaf(dh, v.w, r[4 * k4 + 3]);
                    }
                }
            }
#pragma unroll 1
            for (int turn = 0; turn < 2; ++turn) {
                if (half == turn && jr < H) {
#pragma unroll
                    for (int k = 0; k < 36; ++k) acc[jr * 37 + k] += r[k];
                    acc[jr * 37 + 36] += dw1;
                }
                __syncthreads();
            }
            if (tid < 32) {
                float sg = gt[tid] + gt[tid + 32];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sg += __shfl_xor_sync(0xffffffffu, sg, o);
                db1 += sg;
            }
            __syncthreads();
        }
        if (tid < H) {
            const int j = tid;
            float *dw0 = a.g.w0[l] + (size_t)j * 35;
            for (int k = 0; k < 35; ++k) atomicAdd(dw0 + k, acc[j * 37 + k]);
            atomicAdd(a.g.b0[l] + j, acc[j * 37 + 35]);
            atomicAdd(a.g.w1[l] + j, acc[j * 37 + 36]);
        }
        if (tid == 0) atomicAdd(a.g.b1[l], db1);
    }
}

// ---------------------------------------------------------------------------
// backward 1, tensor-core form (hidden_dim 128, forward ReLU masks given).
// With mask[q][j] = (hidden unit j of point q was positive in the forward)
// and g[q] = dLoss/dpred, the decoder's backward is
//   dh[q][j]  = g[q] mask[q][j] w1[j]
//   dIN[q][c] = sum_j dh[q][j] W[j][c]  = sum_j M[q][j] W1[j][c]
//   dW[j][c]  = sum_q dh[q][j] IN[q][c] = w1[j] E[j][c]
//   dw1[j]    = sum_q g[q] relu(P[q][j]) = sum_c W[j][c] E[j][c]
// with M[q][j] = g[q] mask[q][j], W1[j][c] = w1[j] W[j][c] and
// E[j][c] = sum_q M[q][j] IN[q][c]; IN row of a point = x y z, the 32
// summed features, 1 (the b0 column), zeros; W row j = w0[j][0..34], b0[j].
// Since M = diag(g) Mask with Mask the 1 / 0 ReLU mask, exact in bf16, per
// 128-point tile two products run on tcgen05, each as two bf16 MMAs against
// the hi / lo split of the other operand (relative error about 2^-16 before
// the fp32 accumulation in TMEM):
//   dIN [128 pts x 48]  = Mask [pts x 128 hid] . W1, times g per point in
//                         the epilogue                       (TMEM cols 0..47)
//   E   [128 hid x 48] += Mask^T [hid x pts] . (g IN)        (cols 64..111,
//                         summed over all tiles of a LOD)
// and the hidden layer is never recomputed.  Mask and g IN tiles are
// written once in the K-major core-matrix layout and read by the second
// product through MN-major descriptors (the same 8 x 16 B core matrices: for
// a no-swizzle MN-major operand LBO is the stride between K-adjacent core
// matrices and SBO the stride between MN-adjacent ones).  One operand buffer
// per block (100 KB), two blocks per SM: the next tile's feature sums are
// staged by cp.async while this tile's products and epilogue run, and the
// other block works while one waits.
// ---------------------------------------------------------------------------
namespace bwdtc {
constexpr int kTP = 128, kH = 128, kK1 = 48, kKC1 = kK1 / 8, kKCH = kH / 8;
constexpr int kThreads = 256;
constexpr uint32_t kInBytes = kTP * kK1 * 2;   // 12 KB
constexpr uint32_t kWBytes = kH * kK1 * 2;     // 12 KB
constexpr uint32_t kMBytes = kTP * kH * 2;     // 32 KB
constexpr size_t kIn = 0;                      // g . IN: hi at kIn, lo after it
constexpr size_t kM = kIn + 2 * kInBytes;      // ReLU mask (bf16 1 / 0)
constexpr size_t kWH = kM + kMBytes, kWL = kWH + kWBytes;  // W1 hi / lo
// a tile's feature sums [128][32] f32, rows kStageRow float4 apart: nine,
// so that the eight rows a quarter warp copies or reads fall in eight bank
// groups (eight float4 apart they would share four banks)
constexpr int kStageRow = 9;
constexpr size_t kStage = kWL + kWBytes;
constexpr size_t kStageX = kStage + kTP * kStageRow * 16;  // and positions [128][3] f32
constexpr size_t kBarD = kStageX + kTP * 3 * 4;
constexpr size_t kSlot = kBarD + 8, kAbort = kSlot + 4;
constexpr size_t kSmem = kAbort + 12;
constexpr uint32_t kColDin = 0, kColE = 64, kCols = 128;
constexpr uint32_t kPolls = 1u << 22;
static_assert(kM % 1024 == 0 && kWH % 1024 == 0 && kBarD % 8 == 0, "shared layout alignment");
static_assert(2 * (kSmem + 1024) <= 228 * 1024, "two blocks per SM");
}  // namespace bwdtc


__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 h) { return *reinterpret_cast<uint32_t *>(&h); }

// bf16 hi / lo split of two floats (a in the low half).
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t &hi, uint32_t &lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    hi = bf16x2_bits(h);
    lo = bf16x2_bits(__floats2bfloat162_rn(a - hf.x, b - hf.y));
}

// Column c (0..47, a compile-time index after unrolling) of a point's IN row.
__device__ __forceinline__ float in_column(int c, const float (&xf)[3], const float4 (&fr)[8]) {
    if (c < 3) return xf[c];
    if (c < 35) {
        const float4 v = fr[(c - 3) >> 2];
        const int k = (c - 3) & 3;
        return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
    }
    return c == 35 ? 1.f : 0.f;
}

// Columns 24 HALF .. 24 HALF + 23 of row r of g . IN (hi and lo tiles: the
// point's dLoss/dpred times its decoder input); rows of points past the end
// are zero.
template <int HALF>
__device__ __forceinline__ void fill_in_row(uint8_t *in_hi, uint8_t *in_lo, int r, const float (&xf)[3],
                                            const float4 (&fr)[8], bool valid, float g) {
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
        const int c0 = HALF * 24 + cc * 8;
        uint32_t h[4], lo[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v0 = valid ? g * in_column(c0 + 2 * k, xf, fr) : 0.f;
            const float v1 = valid ? g * in_column(c0 + 2 * k + 1, xf, fr) : 0.f;
            split_bf16x2(v0, v1, h[k], lo[k]);
        }
        const uint32_t off = tc::tile_offset(r, c0, bwdtc::kKC1);
        *reinterpret_cast<uint4 *>(in_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(in_lo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(tc::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Starts the copies of `tile`'s feature sums and positions into the staging
// rows: thread (r, half) copies float4s 4 half .. 4 half + 3 of row r, and
// half 0 the row's x y z.  Rows past the end are not copied.
__device__ __forceinline__ void stage_tile(const BwdArgs &a, int l, int64_t tile, uint8_t *smem, int tid) {
    using namespace bwdtc;
    const int r = tid & (kTP - 1), half = tid >> 7;
    const int64_t q = tile * kTP + r;
    if (q < a.n) {
        const float4 *src = reinterpret_cast<const float4 *>(a.feats + ((int64_t)l * a.n + q) * kC);
        float4 *dst = reinterpret_cast<float4 *>(smem + kStage) + r * kStageRow;
#pragma unroll
        for (int k = 0; k < 4; ++k) cp_async16(dst + 4 * half + k, src + 4 * half + k);
        if (half == 0) {
            float *dx = reinterpret_cast<float *>(smem + kStageX) + r * 3;
#pragma unroll
            for (int k = 0; k < 3; ++k) cp_async4(dx + k, a.x + 3 * q + k);
        }
    }
    cp_async_commit();
}

// IN rows of `tile` (staged by stage_tile, copies complete and visible) into
// IN buffer `buf`: thread (r, half) fills columns 24 half .. 24 half + 23 of
// row r.
__device__ __forceinline__ void fill_in_tile(const BwdArgs &a, int64_t tile, uint8_t *smem, int buf, int tid,
                                             float g) {
    using namespace bwdtc;
    const int r = tid & (kTP - 1), half = tid >> 7;
    const bool valid = tile * kTP + r < a.n;
    const float *sx = reinterpret_cast<const float *>(smem + kStageX) + r * 3;
    const float xf[3] = {sx[0], sx[1], sx[2]};
    float4 fr[8];
    const float4 *sf = reinterpret_cast<const float4 *>(smem + kStage) + r * kStageRow;
#pragma unroll
    for (int k = 0; k < 8; ++k) fr[k] = sf[k];
    uint8_t *hi = smem + kIn + (size_t)(2 * buf) * kInBytes, *lo = hi + kInBytes;
    if (half == 0)
        fill_in_row<0>(hi, lo, r, xf, fr, valid, g);
    else
        fill_in_row<1>(hi, lo, r, xf, fr, valid, g);
}

// Mask row `row` (columns 64 hf .. 64 hf + 63) of buffer `buf`: bf16 1.0
// where the 64 mask bits `bits` are set, else 0 (exact in bf16).
__device__ __forceinline__ void fill_m_row(uint8_t *smem, int buf, int row, int hf, uint2 bits) {
    using namespace bwdtc;
    uint8_t *mt = smem + kM + (size_t)buf * kMBytes;
#pragma unroll
    for (int u = 0; u < 8; ++u) {  // 8 columns per 16-byte store
        const uint32_t b8 = ((u < 4 ? bits.x : bits.y) >> (8 * (u & 3))) & 0xFFu;
        uint32_t h[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            h[k] = ((b8 >> (2 * k)) & 1u ? 0x3F80u : 0u) | ((b8 >> (2 * k + 1)) & 1u ? 0x3F800000u : 0u);
        *reinterpret_cast<uint4 *>(mt + tc::tile_offset(row, 64 * hf + 8 * u, kKCH)) = make_uint4(h[0], h[1], h[2], h[3]);
    }
}

// Thread 0 issues D (+)= A . (B_hi + B_lo) over KSTEPS K steps of 16, for an
// A that bf16 holds exactly (the 1 / 0 mask).
template <int KSTEPS>
__device__ __forceinline__ void mma2(uint32_t d, uint32_t a, uint32_t b_hi, uint32_t b_lo, uint32_t a_lbo,
                                     uint32_t a_sbo, uint32_t a_step, uint32_t b_lbo, uint32_t b_sbo,
                                     uint32_t b_step, uint32_t idesc, bool accumulate) {
    const uint64_t ad0 = tc::smem_desc(a, a_lbo, a_sbo);
    const uint64_t bh = tc::smem_desc(b_hi, b_lbo, b_sbo), bl = tc::smem_desc(b_lo, b_lbo, b_sbo);
#pragma unroll
    for (int t = 0; t < 2; ++t)
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
            // start address >> 4 sits in the descriptor's low bits
            const uint64_t ad = ad0 + (uint64_t)((ks * a_step) >> 4);
            const uint64_t bd = (t == 1 ? bl : bh) + (uint64_t)((ks * b_step) >> 4);
            tc::mma_bf16(d, ad, bd, idesc, (accumulate || t > 0 || ks > 0) ? 1u : 0u);
        }
}

__global__ void __launch_bounds__(bwdtc::kThreads, 2) sdf_bwd_decoder_tc_kernel(const BwdArgs a) {
    using namespace bwdtc;
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    uint8_t *smem = smem_tc;
    uint64_t *barD = reinterpret_cast<uint64_t *>(smem + kBarD);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kAbort);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int sp = warp & 3, hf = warp >> 2;  // TMEM lane quarter, column half
    const int ql = sp * 32 + lane;            // tile row (point, or hidden unit for E) of this thread's TMEM lane

    if (warp == 0) tc::tmem_alloc(slot, kCols);
    if (tid == 0) {
        tc::mbar_init(barD, 1);
        *abort_flag = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t sbase = tc::smem_addr(smem);
    const uint32_t id2 = tc::idesc_bf16_f32(kTP, kK1) | (1u << 16);              // B MN-major
    const uint32_t id3 = tc::idesc_bf16_f32(kH, kK1) | (1u << 15) | (1u << 16);  // A, B MN-major
    const uint32_t trow = (uint32_t)(sp * 32) << 16;
    uint32_t phD = 0;

#pragma unroll 1
    for (int l = 0; l <= a.L && !*abort_flag; ++l) {
        if (!((a.mask >> l) & 1u)) continue;
        int64_t tile = blockIdx.x;
        if (tile * kTP >= a.n) continue;
        // W1 = w1[j] * W[j][c] (hi / lo) for this LOD, and the first tile's rows
        for (int u = tid; u < kH * kKC1; u += kThreads) {
            const int j = u / kKC1, cc = u % kKC1;
            const float w1j = a.m.w1[l][j];
            float v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int c = cc * 8 + k;
                v[k] = w1j * (c < 35 ? a.m.w0[l][j * 35 + c] : c == 35 ? a.m.b0[l][j] : 0.f);
            }
            uint32_t h[4], lo[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) split_bf16x2(v[2 * k], v[2 * k + 1], h[k], lo[k]);
            const uint32_t off = tc::tile_offset(j, cc * 8, kKC1);
            *reinterpret_cast<uint4 *>(smem + kWH + off) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4 *>(smem + kWL + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
        float gsum = 0.f;
        float g_cur = 0.f;  // dLoss/dpred of this thread's row of the current tile
        uint2 rm_cur = make_uint2(0u, 0u);
        stage_tile(a, l, tile, smem, tid);
        {
            const int64_t qg = tile * kTP + ql;
            if (qg < a.n) {
                g_cur = a.gpred[(int64_t)l * a.n + qg];
                rm_cur = reinterpret_cast<const uint2 *>(a.relu + ((int64_t)l * a.n + qg) * (kH / 32))[hf];
            }
        }
        bool first = true;

#pragma unroll 1
        for (; tile * kTP < a.n; tile += gridDim.x) {
            const int64_t next = tile + gridDim.x;
            const bool has_next = next * kTP < a.n;
            // 1. this tile's rows into the operand buffer (its last products
            // completed before the previous epilogue)
            fill_m_row(smem, 0, ql, hf, rm_cur);
            if (hf == 0) gsum += g_cur;
            cp_async_wait_all();
            __syncthreads();
            fill_in_tile(a, tile, smem, 0, tid, g_cur);
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            // 2. the next tile's feature sums and its g and mask start loading
            // while the products run: dIN = g (Mask . W1) (g in the
            // epilogue), E += Mask^T . (g IN)
            float g_next = 0.f;
            uint2 rm_next = make_uint2(0u, 0u);
            if (has_next) {
                stage_tile(a, l, next, smem, tid);
                const int64_t qn = next * kTP + ql;
                if (qn < a.n) {
                    g_next = a.gpred[(int64_t)l * a.n + qn];
                    rm_next = reinterpret_cast<const uint2 *>(a.relu + ((int64_t)l * a.n + qn) * (kH / 32))[hf];
                }
            }
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t mt = sbase + (uint32_t)kM;
                const uint32_t ih = sbase + (uint32_t)kIn, il = ih + kInBytes;
                mma2<kH / 16>(tmem + kColDin, mt, sbase + (uint32_t)kWH, sbase + (uint32_t)kWL, 128, kKCH * 128, 256,
                              kKC1 * 128, 128, 2 * kKC1 * 128, id2, false);
                mma2<kTP / 16>(tmem + kColE, mt, ih, il, kKCH * 128, 128, 2 * kKCH * 128, kKC1 * 128, 128,
                               2 * kKC1 * 128, id3, !first);
                tc::mma_commit(barD);
            }
            first = false;
            // 3. wait for the products, then dLoss/d(feature sum) and the
            // decoder's dLoss/dx of row ql
            if (tid == 0) {
                if (!tc::mbar_wait_bounded(barD, phD, kPolls)) {
                    *abort_flag = 1;
                    atomicExch(&g_train_status, 1);
                }
                phD ^= 1u;
            }
            __syncthreads();
            if (*abort_flag) break;
            tc::fence_after_sync();
            {
                const int64_t qg = tile * kTP + ql;
                float v[32];
                tc::tmem_load32(tmem + trow + kColDin + (uint32_t)(32 * hf), v);
#pragma unroll
                for (int k = 0; k < 32; ++k) v[k] *= g_cur;
                if (qg < a.n) {
                    float *o = a.dfeat + ((int64_t)l * a.n + qg) * kC;
                    if (hf == 0) {
                        if (a.gx) {
                            a.gx[3 * qg] += v[0];
                            a.gx[3 * qg + 1] += v[1];
                            a.gx[3 * qg + 2] += v[2];
                        }
#pragma unroll
                        for (int k = 0; k < 7; ++k)
                            reinterpret_cast<float4 *>(o)[k] =
                                make_float4(v[3 + 4 * k], v[4 + 4 * k], v[5 + 4 * k], v[6 + 4 * k]);
                        o[28] = v[31];
                    } else {
                        o[29] = v[0];
                        o[30] = v[1];
                        o[31] = v[2];
                    }
                }
            }
            g_cur = g_next;
            rm_cur = rm_next;
        }
        if (*abort_flag) break;
        // LOD totals from E (TMEM row j = ql): dW0 = w1 E, db0 = w1 E[:, 35],
        // dw1 = sum_c W E; db1 = sum g
        {
            float v[32];
            tc::tmem_load32(tmem + trow + kColE + (uint32_t)(32 * hf), v);
            const int j = ql;
            const float w1j = a.m.w1[l][j];
            const float *w0r = a.m.w0[l] + j * 35;
            float dw1 = 0.f;
            if (hf == 0) {
#pragma unroll 4
                for (int c = 0; c < 32; ++c) {
                    atomicAdd(a.g.w0[l] + j * 35 + c, w1j * v[c]);
                    dw1 = fmaf(w0r[c], v[c], dw1);
                }
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    atomicAdd(a.g.w0[l] + j * 35 + 32 + c, w1j * v[c]);
                    dw1 = fmaf(w0r[32 + c], v[c], dw1);
                }
                atomicAdd(a.g.b0[l] + j, w1j * v[3]);
                dw1 = fmaf(a.m.b0[l][j], v[3], dw1);
            }
            atomicAdd(a.g.w1[l] + j, dw1);
            if (hf == 0) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) gsum += __shfl_xor_sync(0xffffffffu, gsum, o);
                if (lane == 0) atomicAdd(a.g.b1[l], gsum);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (*abort_flag && tid == 0) {  // let in-flight MMAs finish before the columns are freed
        tc::mma_commit(barD);
        tc::mbar_wait_bounded(barD, phD, kPolls);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------------------
// backward 2: trilinear scatter into the volumes (+ optional dLoss/dx)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void red_add_v4(float *addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Volumes below `smem_levels` are accumulated in shared memory (offsets in
// floats given by soff[l]); the rest go straight to global memory.  A shared
// vertex takes kSV = 33 floats (32 channels and a pad word).
//
// Each warp handles 32 points at a time, cooperatively, in eight passes of
// four points: the eight lanes 8j .. 8j + 7 of pass p own channels
// 4 (lane % 8) .. +3 of point 4p + j.  Within a pass the LODs run from the
// finest down, so each lane carries one running gradient G (suffix sum over
// the mask LODs l >= i of dLoss/d(feature sum l)), loaded as whole 128-byte
// rows; each corner's 32-channel update is one 128-byte vector reduction
// (red.global.add.v4.f32 from eight lanes) or 32 consecutive shared-memory
// atomics.  The eight lanes of a point compute its corner set themselves
// (no shuffles), with the weights formed as (wx * wy) * wz, as in the
// forward.  The loop body stays small: the fully unrolled form (all passes
// of a LOD at once) spent most of its stalls on instruction fetch.
constexpr int kSV = kC + 1;
constexpr int kScatterThreads = 512;
struct ScatterArgs {
    BwdArgs a;
    int smem_levels;
    int soff[NGLOD_MAX_LODS + 1];
};

template <bool kGradX>
__global__ void __launch_bounds__(kScatterThreads, 2) sdf_bwd_scatter_kernel(const ScatterArgs s) {
    extern __shared__ float sacc[];
    const BwdArgs &a = s.a;
    const unsigned FULL = 0xffffffffu;
    const int stot = s.soff[s.smem_levels];
    for (int i = threadIdx.x; i < stot; i += blockDim.x) sacc[i] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, part = lane & 7;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + warp * 32; base < a.n; base += stride) {
        // four points per pass, eight lanes per point (lane: channels 4 part .. +3)
#pragma unroll 1
        for (int p = 0; p < 8; ++p) {
            const int64_t ip = base + 4 * p + (lane >> 3);
            const bool valid = ip < a.n;
            float px = 0.f, py = 0.f, pz = 0.f;
            if (valid) {
                px = a.x[3 * ip];
                py = a.x[3 * ip + 1];
                pz = a.x[3 * ip + 2];
            }
            float4 G = make_float4(0.f, 0.f, 0.f, 0.f);
            float gxv[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
            for (int l = a.L; l >= 0; --l) {
                // G: dLoss / d(feature sum of LODs 0..l) = sum of dfeat over decoded LODs >= l
                if (valid && ((a.mask >> l) & 1u)) {
                    const float4 v = reinterpret_cast<const float4 *>(a.dfeat + ((int64_t)l * a.n + ip) * kC)[part];
                    G.x += v.x;
                    G.y += v.y;
                    G.z += v.z;
                    G.w += v.w;
                }
                // the point's corner set at LOD l, in every lane of the point
                const int sd = volume_side(a.m, l);
                const float sm1 = (float)(sd - 1);
                const float rx = ((px + 1.f) / 2.f) * sm1;
                const float ry = ((py + 1.f) / 2.f) * sm1;
                const float rz = ((pz + 1.f) / 2.f) * sm1;
                const float ix = fminf(sm1, fmaxf(rx, 0.f));
                const float iy = fminf(sm1, fmaxf(ry, 0.f));
                const float iz = fminf(sm1, fmaxf(rz, 0.f));
                const float x0 = floorf(ix), y0 = floorf(iy), z0 = floorf(iz);
                const float w6[6] = {(x0 + 1.f) - ix, ix - x0, (y0 + 1.f) - iy, iy - y0, (z0 + 1.f) - iz, iz - z0};
                const int xi = (int)x0, yi = (int)y0, zi = (int)z0;
                const float w[8] = {w6[0] * w6[2] * w6[4], w6[1] * w6[2] * w6[4], w6[0] * w6[3] * w6[4],
                                    w6[1] * w6[3] * w6[4], w6[0] * w6[2] * w6[5], w6[1] * w6[2] * w6[5],
                                    w6[0] * w6[3] * w6[5], w6[1] * w6[3] * w6[5]};
                const int v0 = (zi * sd + yi) * sd + xi;
                const int ox = xi + 1 < sd ? 1 : 0;
                const int oy = yi + 1 < sd ? sd : 0;
                const int oz = zi + 1 < sd ? sd * sd : 0;
                const int vtx[8] = {v0, v0 + ox, v0 + oy, v0 + oy + ox, v0 + oz, v0 + oz + ox, v0 + oz + oy, v0 + oz + oy + ox};
                if (valid) {
                    if (l < s.smem_levels) {
                        float *gbase = sacc + s.soff[l] + 4 * part;
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            float *dst = gbase + vtx[k] * kSV;
                            atomicAdd(dst, G.x * w[k]);
                            atomicAdd(dst + 1, G.y * w[k]);
                            atomicAdd(dst + 2, G.z * w[k]);
                            atomicAdd(dst + 3, G.w * w[k]);
                        }
                    } else {
                        float *gbase = a.g.grid[l] + 4 * part;
#pragma unroll
                        for (int k = 0; k < 8; ++k)
                            red_add_v4(gbase + (size_t)vtx[k] * kC, G.x * w[k], G.y * w[k], G.z * w[k], G.w * w[k]);
                    }
                }
                if (kGradX) {
                    // d(sample)/du per corner: -/+ the product of the other two axes' weights
                    // (PyTorch's grid_sampler_3d backward), times (s-1)/2, zero where clamped.
                    const float4 *fm = reinterpret_cast<const float4 *>(a.m.grid[l]);
                    float dot[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const float4 u = __ldg(fm + (size_t)vtx[k] * (kC / 4) + part);
                        float t = G.x * u.x;
                        t = fmaf(G.y, u.y, t);
                        t = fmaf(G.z, u.z, t);
                        t = fmaf(G.w, u.w, t);
                        t += __shfl_xor_sync(FULL, t, 1);
                        t += __shfl_xor_sync(FULL, t, 2);
                        t += __shfl_xor_sync(FULL, t, 4);
                        dot[k] = t;
                    }
                    const float wx0 = w6[0], wx1 = w6[1], wy0 = w6[2], wy1 = w6[3], wz0 = w6[4], wz1 = w6[5];
                    float gix = 0.f, giy = 0.f, giz = 0.f;
                    gix += -dot[0] * wy0 * wz0 + dot[1] * wy0 * wz0 - dot[2] * wy1 * wz0 + dot[3] * wy1 * wz0;
                    gix += -dot[4] * wy0 * wz1 + dot[5] * wy0 * wz1 - dot[6] * wy1 * wz1 + dot[7] * wy1 * wz1;
                    giy += -dot[0] * wx0 * wz0 - dot[1] * wx1 * wz0 + dot[2] * wx0 * wz0 + dot[3] * wx1 * wz0;
                    giy += -dot[4] * wx0 * wz1 - dot[5] * wx1 * wz1 + dot[6] * wx0 * wz1 + dot[7] * wx1 * wz1;
                    giz += -dot[0] * wx0 * wy0 - dot[1] * wx1 * wy0 - dot[2] * wx0 * wy1 - dot[3] * wx1 * wy1;
                    giz += dot[4] * wx0 * wy0 + dot[5] * wx1 * wy0 + dot[6] * wx0 * wy1 + dot[7] * wx1 * wy1;
                    const float half = sm1 / 2.f;
                    gxv[0] += (rx <= 0.f || rx >= sm1) ? 0.f : gix * half;
                    gxv[1] += (ry <= 0.f || ry >= sm1) ? 0.f : giy * half;
                    gxv[2] += (rz <= 0.f || rz >= sm1) ? 0.f : giz * half;
                }
            }
            if (kGradX && part == 0 && valid) {
                a.gx[3 * ip] += gxv[0];
                a.gx[3 * ip + 1] += gxv[1];
                a.gx[3 * ip + 2] += gxv[2];
            }
        }
    }
    __syncthreads();
    for (int l = 0; l < s.smem_levels; ++l) {
        const int nq = (s.soff[l + 1] - s.soff[l]) / kSV * (kC / 4);  // vertices x channel quads
        float *dst = a.g.grid[l];
        const float *src = sacc + s.soff[l];
        for (int i = threadIdx.x; i < nq; i += blockDim.x) {
            const int v = i / (kC / 4), c = 4 * (i % (kC / 4));
            const float *r = src + v * kSV + c;
            red_add_v4(dst + (size_t)v * kC + c, r[0], r[1], r[2], r[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// L2 loss of Trainer.step_geometry and its gradient in one pass
// ---------------------------------------------------------------------------
// Error-free transformations in float32 (Knuth's TwoSum; Dekker's product
// with one FMA), in round-to-nearest intrinsics so that no step is fused.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (ah, al) += (xh, xl) for float-float values of one sign: about 2^-46
// relative error per addition, ah the float nearest to the pair's sum.
__device__ __forceinline__ void ff_add(float &ah, float &al, float xh, float xl) {
    float s, e;
    two_sum(ah, xh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, xl));
    ah = __fadd_rn(s, e);
    al = __fsub_rn(e, __fsub_rn(ah, s));
}

// preds [rows][n], gts [n]: loss = sum over l in mask, q of (preds - gts)^2
// / n to float64 accuracy; grad[l][q] = 2 (preds - gts) / n for l in mask,
// else 0.  One thread takes a point and loads its gt and every row's
// prediction before using them (rows <= NGLOD_MAX_LODS loads in flight).
// The squares are summed as float-float pairs in float32 arithmetic, whose
// rate is far above float64's on this part: p - g = s + e exactly (TwoSum),
// (p - g)^2 = s*s (an exact pair through one FMA) + 2 s e, dropping e*e
// (below 2^-48 of s*s), so a term is exact to about 2^-46 while
// 2^-63 < |p - g| < 2^63.  Each warp's pair goes to float64 once; block
// sums in float64, one double atomic per block.
__global__ void __launch_bounds__(256) l2_loss_kernel(const float *__restrict__ preds, const float *__restrict__ gts,
                                                      int64_t n, int rows, uint32_t mask, double *loss,
                                                      float *__restrict__ grad) {
    __shared__ double part[8];
    const float scale = 2.f / (float)n;
    float ah = 0.f, al = 0.f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const float g = gts[q];
        float p[NGLOD_MAX_LODS];
#pragma unroll
        for (int l = 0; l < NGLOD_MAX_LODS; ++l) p[l] = l < rows ? preds[(int64_t)l * n + q] : 0.f;
#pragma unroll
        for (int l = 0; l < NGLOD_MAX_LODS; ++l) {
            if (l >= rows) break;
            const bool on = (mask >> l) & 1u;
            if (on) {
                float d, e;
                two_sum(p[l], -g, d, e);
                const float sq = __fmul_rn(d, d);
                const float sq_err = fmaf(d, d, -sq);
                ff_add(ah, al, sq, __fadd_rn(sq_err, __fmul_rn(__fmul_rn(2.f, d), e)));
            }
            grad[(int64_t)l * n + q] = on ? (p[l] - g) * scale : 0.f;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float xh = __shfl_xor_sync(0xffffffffu, ah, o);
        const float xl = __shfl_xor_sync(0xffffffffu, al, o);
        ff_add(ah, al, xh, xl);
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part[warp] = (double)ah + (double)al;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicAdd(loss, t / (double)n);
    }
}

// ---------------------------------------------------------------------------
// Adam
// ---------------------------------------------------------------------------
// One element of the update (torch.optim.Adam's single-tensor order).
__device__ __forceinline__ void adam_update(float &p, float g, float &m, float &v, float lr_over_bc1, float beta2,
                                            float one_m_b1, float one_m_b2, float bc2_sqrt, float eps, float wd) {
    if (wd != 0.f) g = g + wd * p;
    // torch.lerp with weight < 0.5: m + w * (g - m)
    m = m + one_m_b1 * (g - m);
    v = v * beta2;
    v = v + (one_m_b2 * g) * g;
    const float denom = sqrtf(v) / bc2_sqrt + eps;
    p = p + (-lr_over_bc1) * (m / denom);
}

// blockIdx.y selects the tensor.  Tensors whose four arrays start on 16-byte
// boundaries go four elements per thread and access; the rest of each
// tensor (its last numel % 4 elements, or all of an unaligned one) one.
__global__ void __launch_bounds__(256) adam_kernel(const nglod_adam_tensor *__restrict__ tab, float lr_over_bc1,
                                                   float beta2, float one_m_b1, float one_m_b2, float bc2_sqrt,
                                                   float eps, float wd) {
    const nglod_adam_tensor t = tab[blockIdx.y];
    const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const uintptr_t bits = reinterpret_cast<uintptr_t>(t.param) | reinterpret_cast<uintptr_t>(t.grad) |
                           reinterpret_cast<uintptr_t>(t.exp_avg) | reinterpret_cast<uintptr_t>(t.exp_avg_sq);
    const int64_t nv = (bits & 15u) == 0 ? t.numel / 4 : 0;
    for (int64_t i = first; i < nv; i += stride) {
        const float4 g = reinterpret_cast<const float4 *>(t.grad)[i];
        float4 p = reinterpret_cast<const float4 *>(t.param)[i];
        float4 m = reinterpret_cast<const float4 *>(t.exp_avg)[i];
        float4 v = reinterpret_cast<const float4 *>(t.exp_avg_sq)[i];
        adam_update(p.x, g.x, m.x, v.x, lr_over_bc1, beta2, one_m_b1, one_m_b2, bc2_sqrt, eps, wd);
        adam_update(p.y, g.y, m.y, v.y, lr_over_bc1, beta2, one_m_b1, one_m_b2, bc2_sqrt, eps, wd);
        adam_update(p.z, g.z, m.z, v.z, lr_over_bc1, beta2, one_m_b1, one_m_b2, bc2_sqrt, eps, wd);
        adam_update(p.w, g.w, m.w, v.w, lr_over_bc1, beta2, one_m_b1, one_m_b2, bc2_sqrt, eps, wd);
        reinterpret_cast<float4 *>(t.exp_avg)[i] = m;
        reinterpret_cast<float4 *>(t.exp_avg_sq)[i] = v;
        reinterpret_cast<float4 *>(t.param)[i] = p;
    }
    for (int64_t i = 4 * nv + first; i < t.numel; i += stride) {
        float p = t.param[i], m = t.exp_avg[i], v = t.exp_avg_sq[i];
        adam_update(p, t.grad[i], m, v, lr_over_bc1, beta2, one_m_b1, one_m_b2, bc2_sqrt, eps, wd);
        t.exp_avg[i] = m;
        t.exp_avg_sq[i] = v;
        t.param[i] = p;
    }
}

}  // namespace nglod

using namespace nglod;

static int lod_mask_top(uint32_t mask) {
    int L = -1;
    for (int l = 0; l < NGLOD_MAX_LODS; ++l)
        if ((mask >> l) & 1u) L = l;
    return L;
}

extern "C" int nglod_sdf_fwd_train(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                                   float *preds, float *feats, uint32_t *relu_masks, nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr, NGLOD_ERR_INVALID, "model is null");
    const int L = lod_mask_top(lod_mask);
    NGLOD_REQUIRE(L >= 0 && L < model->num_lods && (lod_mask >> NGLOD_MAX_LODS) == 0, NGLOD_ERR_INVALID,
                  "lod_mask=0x%x selects no LOD or a LOD >= num_lods=%d", lod_mask, model->num_lods);
    NGLOD_TRY(check_model(model, L));
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && preds && feats, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(feats, 16), NGLOD_ERR_ALIGN, "feats must be 16-byte aligned");
    NGLOD_REQUIRE(!relu_masks || aligned(relu_masks, 16), NGLOD_ERR_ALIGN, "relu_masks must be 16-byte aligned");
    if (model->hidden_dim == fwdtc::kH && relu_masks) {
        // tensor-core form: two 256-thread blocks per SM
        NGLOD_TRY(prepare_smem(sdf_fwd_train_tc_kernel, fwdtc::kSmem));
        const int64_t pairs = (n + fwdtc::kThreads - 1) / fwdtc::kThreads;
        const int64_t cap = (int64_t)num_sms() * 2;
        sdf_fwd_train_tc_kernel<<<(int)(pairs < cap ? pairs : cap), fwdtc::kThreads, fwdtc::kSmem,
                                  (cudaStream_t)stream>>>(*model, x, n, L, lod_mask, preds, feats, relu_masks);
        return launch_status("nglod_sdf_fwd_train");
    }
    const int threads = kFwdTrainThreads;
    // staged decoders, then one [32][kTRow] float transpose buffer per warp
    const size_t smem = (size_t)(L + 1) * decoder_f4(model->hidden_dim) * sizeof(float4) +
                        (size_t)threads * kTRow * sizeof(float);
    auto k = relu_masks ? sdf_fwd_train_kernel<true> : sdf_fwd_train_kernel<false>;
    NGLOD_TRY(prepare_smem(k, smem));
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = resident_blocks(k, threads, smem);
    k<<<(int)(want < cap ? want : cap), threads, smem, (cudaStream_t)stream>>>(*model, x, n, L, lod_mask, preds,
                                                                             feats, relu_masks);
    return launch_status("nglod_sdf_fwd_train");
}

extern "C" int nglod_sdf_bwd(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                             const float *grad_preds, const float *feats, const uint32_t *relu_masks,
                             float *dfeat_scratch, const nglod_dense_grads *grads, float *grad_x,
                             nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr && grads != nullptr, NGLOD_ERR_INVALID, "model or grads is null");
    const int L = lod_mask_top(lod_mask);
    NGLOD_REQUIRE(L >= 0 && L < model->num_lods && (lod_mask >> NGLOD_MAX_LODS) == 0, NGLOD_ERR_INVALID,
                  "lod_mask=0x%x selects no LOD or a LOD >= num_lods=%d", lod_mask, model->num_lods);
    NGLOD_TRY(check_model(model, L));
    NGLOD_REQUIRE(model->hidden_dim <= kBT, NGLOD_ERR_UNSUPPORTED, "backward built for hidden_dim <= %d", kBT);
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && grad_preds && feats && dfeat_scratch, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(feats, 16) && aligned(dfeat_scratch, 16), NGLOD_ERR_ALIGN,
                  "feats and dfeat_scratch must be 16-byte aligned");
    NGLOD_REQUIRE(!relu_masks || aligned(relu_masks, 16), NGLOD_ERR_ALIGN, "relu_masks must be 16-byte aligned");
    for (int l = 0; l <= L; ++l) {
        NGLOD_REQUIRE(grads->grid[l] && aligned(grads->grid[l], 16), NGLOD_ERR_INVALID,
                      "volume gradient %d is null or not 16-byte aligned", l);
        if ((lod_mask >> l) & 1u)
            NGLOD_REQUIRE(grads->w0[l] && grads->b0[l] && grads->w1[l] && grads->b1[l], NGLOD_ERR_INVALID,
                          "decoder gradient %d has a null pointer", l);
    }
    BwdArgs a;
    a.m = *model;
    a.g = *grads;
    a.x = x;
    a.n = n;
    a.mask = lod_mask;
    a.L = L;
    a.gpred = grad_preds;
    a.feats = feats;
    a.relu = relu_masks;
    a.dfeat = dfeat_scratch;
    a.gx = grad_x;

    if (model->hidden_dim == bwdtc::kH && relu_masks) {
        // tensor-core form: two blocks of 256 threads per SM
        NGLOD_TRY(prepare_smem(sdf_bwd_decoder_tc_kernel, bwdtc::kSmem));
        const int64_t tiles = (n + bwdtc::kTP - 1) / bwdtc::kTP;
        const int64_t cap1 = (int64_t)num_sms() * 2;
        sdf_bwd_decoder_tc_kernel<<<(int)(tiles < cap1 ? tiles : cap1), bwdtc::kThreads, bwdtc::kSmem,
                                    (cudaStream_t)stream>>>(a);
    } else {
        const size_t smem1 = bwd_decoder_smem(model->hidden_dim);
        NGLOD_TRY(prepare_smem(sdf_bwd_decoder_kernel, smem1));
        const int64_t tiles = (n + kBP - 1) / kBP;
        const int64_t cap1 = resident_blocks(sdf_bwd_decoder_kernel, kBThreads, smem1);
        sdf_bwd_decoder_kernel<<<(int)(tiles < cap1 ? tiles : cap1), kBThreads, smem1, (cudaStream_t)stream>>>(a);
    }
    NGLOD_TRY(launch_status("nglod_sdf_bwd (decoder)"));

    ScatterArgs s;
    s.a = a;
    s.smem_levels = 0;
    s.soff[0] = 0;
    const int budget = 112 * 1024 / (int)sizeof(float);  // leave room for two blocks per SM
    for (int l = 0; l <= L; ++l) {
        const int side = (1 << (l + model->base_lod)) + 1;
        const int cnt = side * side * side * kSV;
        if (s.soff[l] + cnt > budget) break;
        s.soff[l + 1] = s.soff[l] + cnt;
        s.smem_levels = l + 1;
    }
    const size_t smem2 = (size_t)s.soff[s.smem_levels] * sizeof(float);
    const int threads = kScatterThreads;
    const int64_t want = (n + threads - 1) / threads;
    if (grad_x) {
        auto k = sdf_bwd_scatter_kernel<true>;
        NGLOD_TRY(prepare_smem(k, smem2));
        const int64_t cap = resident_blocks(k, threads, smem2);
        k<<<(int)(want < cap ? want : cap), threads, smem2, (cudaStream_t)stream>>>(s);
    } else {
        auto k = sdf_bwd_scatter_kernel<false>;
        NGLOD_TRY(prepare_smem(k, smem2));
        const int64_t cap = resident_blocks(k, threads, smem2);
        k<<<(int)(want < cap ? want : cap), threads, smem2, (cudaStream_t)stream>>>(s);
    }
    return launch_status("nglod_sdf_bwd (scatter)");
}

extern "C" int nglod_adam_step(const nglod_adam_tensor *tensors, int32_t count, int64_t max_numel, float lr,
                               float beta1, float beta2, float eps, float weight_decay, int64_t step,
                               nglod_stream_t stream) {
    NGLOD_REQUIRE(count >= 0 && count <= 65535, NGLOD_ERR_INVALID, "count=%d outside [0, 65535]", count);
    NGLOD_REQUIRE(step >= 1, NGLOD_ERR_INVALID, "step=%lld: the first step is 1", (long long)step);
    if (count == 0 || max_numel <= 0) return NGLOD_OK;
    NGLOD_REQUIRE(tensors != nullptr, NGLOD_ERR_INVALID, "tensor table is null");
    const double bc1 = 1.0 - pow((double)beta1, (double)step);
    const double bc2 = 1.0 - pow((double)beta2, (double)step);
    const int threads = 256;
    int64_t bx = (max_numel + 4 * threads - 1) / (4 * threads);
    const int64_t cap = (int64_t)num_sms() * 8;
    if (bx > cap) bx = cap;
    dim3 grid((unsigned)bx, (unsigned)count);
    adam_kernel<<<grid, threads, 0, (cudaStream_t)stream>>>(tensors, (float)((double)lr / bc1), beta2,
                                                            (float)(1.0 - (double)beta1), (float)(1.0 - (double)beta2),
                                                            (float)sqrt(bc2), eps, weight_decay);
    return launch_status("nglod_adam_step");
}

// ---------------------------------------------------------------------------
// Backward for callers that cannot allocate device memory
// ---------------------------------------------------------------------------
// nglod_sdf_bwd needs a per-point scratch buffer (dLoss/d(feature sum) for
// every point and LOD) that the caller allocates.  Some callers cannot call
// cudaMalloc at all: a plugin or engine whose GPU memory belongs to a host
// runtime that hands out only the buffers it manages (inputs and outputs),
// or a process whose allocator is locked after start-up.  For them,
// nglod_sdf_bwd_noalloc takes that scratch from a fixed array compiled into
// this library, so the call needs nothing beyond its inputs and outputs and
// itself calls no allocator.
//
// The array is 16 MiB on every GPU that loads the library and stays there
// until the process exits.  It holds (L+1) * n * 32 floats, so one call
// covers at most 131,072 point-LODs (26,214 points when all 5 LODs of the
// reference architecture carry a loss); larger calls are rejected.  All calls
// share the one array: calls that run at the same time on the GPU (different
// streams, or different host threads on one device) overwrite each other's
// scratch and must be serialised by the caller.  Nothing in the array has to
// start at zero: each call writes every element it later reads.
namespace nglod {

constexpr size_t kNoAllocScratchFloats = (size_t)4 << 20;  // 16 MiB of float32

static __device__ __align__(256) float g_bwd_noalloc_scratch[kNoAllocScratchFloats];

// The array has one instance per CUDA context that loads this module, at
// that context's address.  The address is cached per context, keyed by the
// CUcontext handle (read through the runtime's driver entry point, so the
// library needs no link to the driver).  Outside stream capture every call
// looks the address up again with cudaGetSymbolAddress and refreshes the
// cache, so a context destroyed and created again at the same handle
// (cudaDeviceReset, cuCtxDestroy + cuCtxCreate) is picked up by the next
// call.  A call made while its stream is capturing uses the cache only and
// fails if the current context has none, so the first call in every context
// -- and the first call after a reset -- must come before any capture.
constexpr int kNoAllocMaxContexts = 64;
struct NoAllocSlot {
    CUcontext ctx;
    float *addr;
};
static NoAllocSlot g_bwd_noalloc_slots[kNoAllocMaxContexts] = {};
static std::mutex g_bwd_noalloc_mutex;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);

static int current_context(CUcontext *ctx) {
    static CtxGetCurrentFn fn = nullptr;
    if (fn == nullptr) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        NGLOD_TRY(cuda_status(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q),
                              "nglod_sdf_bwd_noalloc: cudaGetDriverEntryPointByVersion"));
        NGLOD_REQUIRE(q == cudaDriverEntryPointSuccess && p != nullptr, NGLOD_ERR_CUDA,
                      "nglod_sdf_bwd_noalloc: cuCtxGetCurrent not found in the driver");
        fn = reinterpret_cast<CtxGetCurrentFn>(p);
    }
    *ctx = nullptr;
    NGLOD_REQUIRE(fn(ctx) == CUDA_SUCCESS && *ctx != nullptr, NGLOD_ERR_CUDA,
                  "nglod_sdf_bwd_noalloc: no current CUDA context");
    return NGLOD_OK;
}

// Device address of the array in the current context (the symbol's host-side
// name is not a device address and must never be passed to a kernel).
static int noalloc_scratch_address(cudaStream_t stream, float **out) {
    // a runtime call first: it makes the current device's context current
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    NGLOD_TRY(cuda_status(cudaStreamIsCapturing(stream, &cs), "nglod_sdf_bwd_noalloc: cudaStreamIsCapturing"));
    CUcontext ctx = nullptr;
    NGLOD_TRY(current_context(&ctx));
    std::lock_guard<std::mutex> lock(g_bwd_noalloc_mutex);
    int slot = -1, free_slot = -1;
    for (int i = 0; i < kNoAllocMaxContexts; ++i) {
        if (g_bwd_noalloc_slots[i].ctx == ctx) slot = i;
        if (g_bwd_noalloc_slots[i].ctx == nullptr && free_slot < 0) free_slot = i;
    }
    if (cs == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        NGLOD_TRY(cuda_status(cudaGetSymbolAddress(&p, g_bwd_noalloc_scratch),
                              "nglod_sdf_bwd_noalloc: cudaGetSymbolAddress"));
        if (slot < 0) slot = free_slot;
        NGLOD_REQUIRE(slot >= 0, NGLOD_ERR_UNSUPPORTED, "nglod_sdf_bwd_noalloc: more than %d CUDA contexts",
                      kNoAllocMaxContexts);
        g_bwd_noalloc_slots[slot] = {ctx, static_cast<float *>(p)};
    } else {
        NGLOD_REQUIRE(slot >= 0, NGLOD_ERR_INVALID,
                      "nglod_sdf_bwd_noalloc: first call in this CUDA context made during stream capture; "
                      "call it once outside capture first");
    }
    *out = g_bwd_noalloc_slots[slot].addr;
    return NGLOD_OK;
}

}  // namespace nglod

extern "C" int nglod_sdf_bwd_noalloc(const nglod_dense_model *model, const float *x, int64_t n,
                                     uint32_t lod_mask, const float *grad_preds, const float *feats,
                                     const uint32_t *relu_masks, const nglod_dense_grads *grads, float *grad_x,
                                     nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr && grads != nullptr, NGLOD_ERR_INVALID, "model or grads is null");
    const int L = lod_mask_top(lod_mask);
    NGLOD_REQUIRE(L >= 0 && L < model->num_lods && (lod_mask >> NGLOD_MAX_LODS) == 0, NGLOD_ERR_INVALID,
                  "lod_mask=0x%x selects no LOD or a LOD >= num_lods=%d", lod_mask, model->num_lods);
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    NGLOD_REQUIRE(model->feature_dim == kC, NGLOD_ERR_UNSUPPORTED, "feature_dim=%d not built (only %d)",
                  model->feature_dim, kC);
    const size_t per_point = (size_t)(L + 1) * kC;
    NGLOD_REQUIRE((size_t)n <= kNoAllocScratchFloats / per_point, NGLOD_ERR_CAPACITY,
                  "nglod_sdf_bwd_noalloc: n=%lld points x %d LODs needs %zu scratch floats, the built-in "
                  "array holds %zu (16 MiB): at most %zu points for this lod_mask; use nglod_sdf_bwd with "
                  "caller-provided scratch for larger batches",
                  (long long)n, L + 1, (size_t)n * per_point, kNoAllocScratchFloats,
                  kNoAllocScratchFloats / per_point);
    if (n == 0) return NGLOD_OK;
    float *scratch = nullptr;
    NGLOD_TRY(noalloc_scratch_address((cudaStream_t)stream, &scratch));
    return nglod_sdf_bwd(model, x, n, lod_mask, grad_preds, feats, relu_masks, scratch, grads, grad_x, stream);
}

extern "C" int nglod_train_status(int32_t *status_out) {
    NGLOD_REQUIRE(status_out != nullptr, NGLOD_ERR_INVALID, "null pointer argument");
    int32_t v = 0;
    const int32_t zero = 0;
    NGLOD_TRY(cuda_status(cudaMemcpyFromSymbol(&v, g_train_status, sizeof(v)), "nglod_train_status: read"));
    NGLOD_TRY(cuda_status(cudaMemcpyToSymbol(g_train_status, &zero, sizeof(zero)), "nglod_train_status: reset"));
    *status_out = v;
    return NGLOD_OK;
}

extern "C" int nglod_l2_loss(const float *preds, const float *gts, int64_t n, int32_t rows, uint32_t lod_mask,
                             double *loss_out, float *grad_preds, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && rows >= 1 && rows <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID, "n=%lld rows=%d",
                  (long long)n, rows);
    NGLOD_REQUIRE(loss_out != nullptr, NGLOD_ERR_INVALID, "loss_out is null");
    cudaStream_t s = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemsetAsync(loss_out, 0, sizeof(double), s), "nglod_l2_loss memset"));
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(preds && gts && grad_preds, NGLOD_ERR_INVALID, "null pointer argument");
    const int threads = 256;
    const int64_t want = (n + threads - 1) / threads, cap = (int64_t)num_sms() * 8;
    l2_loss_kernel<<<(int)(want < cap ? want : cap), threads, 0, s>>>(preds, gts, n, rows, lod_mask, loss_out,
                                                                      grad_preds);
    return launch_status("nglod_l2_loss");
}
