// Dense NGLOD path, float32: ray/box entry, fused LOD gather + decoder, and a
// persistent sphere tracer.  Building blocks live in dense_common.cuh.
#include "dense_common.cuh"
#include "f32_tile.cuh"

namespace nglod {

// ---------------------------------------------------------------------------
// sdf forward
// ---------------------------------------------------------------------------
// Each warp evaluates 32 points at a time (lane i owns point base + i): the
// LOD sums are gathered cooperatively (gather_warp_add_f32), handed to the
// point owners through a per-warp shared buffer placed after the staged
// decoders, and each lane decodes its own point.
template <bool kAll>
__global__ void __launch_bounds__(256, kAll ? 2 : 3) sdf_fwd_f32_kernel(const nglod_dense_model m, const float *__restrict__ x,
                                                          int64_t n, int L, float *__restrict__ out) {
    extern __shared__ float4 smem[];
    const int H = m.hidden_dim;
    const int dstride = decoder_f4(H);
    const int first = kAll ? 0 : L;
    for (int l = first; l <= L; ++l) stage_decoder(smem + (l - first) * dstride, m, l);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *sT = reinterpret_cast<float *>(smem + (L - first + 1) * dstride) + warp * 32 * kTRow;
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
        float f[kC];
#pragma unroll 1
        for (int l = 0; l <= L; ++l) {
            gather_warp_add_f32(static_cast<const float *>(m.grid[l]), volume_side(m, l), px, py, pz, lane, acc);
            if (kAll) {
                warp_sums_to_points(sT, lane, acc, f);
                const float o = decode_f32(smem + l * dstride, H, px, py, pz, f);
                if (i < n) out[(int64_t)l * n + i] = o;
            }
        }
        if (!kAll) {
            warp_sums_to_points(sT, lane, acc, f);
            const float o = decode_f32(smem, H, px, py, pz, f);
            if (i < n) out[i] = o;
        }
    }
}

// ---------------------------------------------------------------------------
// tensor-core decode of the float32 tracer (single LOD, hidden 128)
// ---------------------------------------------------------------------------
// The same gather and LOD sum as sdf_fwd_f32_kernel (gather_warp_add_f32, in
// float32), then the decoder's first layer on tcgen05 as split-TF32 products
// over big / small parts of both operands (f32_tile.cuh, tf32_tile.cuh:
// relative error about 2^-21 of sum |w x|, the size of float32's rounding),
// accumulated in TMEM; the ReLU and the 128 -> 1 layer are a float32
// epilogue per point.
//
// A block of eight warps decodes two 128-point tiles per iteration against
// one staged weight side: warps 0-3 fill tile 0, warps 4-7 tile 1 (warp w,
// lane i owns point 32 w + i of the block's 256), one thread issues both
// tiles' 28 MMAs, and each warp reads its rows back from the TMEM lanes of
// its quadrant (warp % 4) in its tile's 128 columns.  Two blocks per SM hold
// 2 x 256 TMEM columns, the SM's 512.  The point query runs the same rows,
// products and epilogue in the persistent kernel below.
namespace f32tc {
using f32tile::kTP;
using f32tile::kH;
using f32tile::kK;
using f32tile::kKC;
using f32tile::kTileA;
using f32tile::kWBytes;
constexpr int kTiles = 2;                     // tiles per block iteration
constexpr int kThreads = kTP * kTiles;        // 256
constexpr size_t kA = 0;                      // tile h at kA + h kTileA
constexpr size_t kW = kTiles * kTileA;
constexpr size_t kW1 = kW + kWBytes;          // w1 [kH]
constexpr size_t kBar = kW1 + kH * 4;
constexpr size_t kSlot = kBar + 8, kAbort = kSlot + 4;
constexpr size_t kSmem = kAbort + 12;
constexpr uint32_t kCols = kTiles * kH;       // TMEM columns per block
static_assert(kW % 1024 == 0 && kBar % 8 == 0, "swizzled tiles start on 1024-byte boundaries");
static_assert(2 * (kSmem + 1024) <= 228 * 1024, "two blocks per SM");
}  // namespace f32tc

// Set by a tensor-core wait of the float32 query or tracer that gave up; read and
// cleared by nglod_dense_status.
__device__ int g_dense_status = 0;
// Bound of that wait (host side, all devices): kPolls unless a test of the
// error path lowers it.
static uint32_t g_f32tc_wait_polls = 1u << 22;

// Block set-up of the tensor-core float32 decode: LOD L's weight side and
// w1, TMEM columns, the barrier.  Returns the TMEM base address.
__device__ __forceinline__ uint32_t f32tc_setup(const nglod_dense_model &m, int L, uint8_t *sm, int tid) {
    using namespace f32tc;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + kSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    stage_tf32_decoder(m, L, sm + kW, sm + kW1, tid, kThreads);
    if ((tid >> 5) == 0) tc::tmem_alloc(slot, kCols);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        *abort_flag = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    return *slot;
}

// The sdf of the block's 256 points at LOD L, thread tid owning point
// (px, py, pz) (warp w fills row 32 (w % 4) + lane of tile w / 4): the
// warp-cooperative gather and LOD sum, the tile rows, one thread's 28
// split-TF32 MMAs for both tiles, and this thread's float32 epilogue.  Every
// thread of the block calls it; false (for all of them) if the bounded
// tensor-core wait gave up, which also sets g_dense_status.
__device__ __forceinline__ bool f32tc_decode(const nglod_dense_model &m, int L, float px, float py, float pz,
                                             uint8_t *sm, uint32_t tmem, uint32_t &phase, uint32_t polls,
                                             float &out) {
    using namespace f32tc;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int half = warp >> 2, quad = warp & 3;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBar);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    const float *sw1 = reinterpret_cast<const float *>(sm + kW1);
    // 1. gather: LOD sum of the warp's 32 points, written as tile rows
    float4 acc[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) acc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
    for (int l = 0; l <= L; ++l)
        gather_warp_add_f32(static_cast<const float *>(m.grid[l]), volume_side(m, l), px, py, pz, lane, acc);
    store_point_rows(sm + kA + (size_t)half * kTileA, quad * 32, lane, acc, px, py, pz);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // 2. one thread issues both tiles' first layers
    if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t sbase = tc::smem_addr(sm);
#pragma unroll
        for (int h = 0; h < kTiles; ++h)
            issue_first_layer(tmem + (uint32_t)(h * kH), sbase + (uint32_t)(kA + h * kTileA), sbase + (uint32_t)kW);
        tc::mma_commit(bar);
        if (!tc::mbar_wait_bounded(bar, phase, polls)) {
            *abort_flag = 1;
            atomicExch(&g_dense_status, 1);
        }
    }
    __syncthreads();
    if (*abort_flag) return false;
    phase ^= 1u;
    tc::fence_after_sync();
    // 3. epilogue: ReLU and the 128 -> 1 layer on this thread's TMEM row
    const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * kH);
    out = relu_dot_w1_f32(taddr, sw1) + m.b1[L][0];
    tc::fence_before_sync();
    return true;
}

// Block teardown: lets an issued product finish after a wait gave up, then
// frees the TMEM columns.
__device__ __forceinline__ void f32tc_teardown(uint8_t *sm, uint32_t tmem, uint32_t phase) {
    using namespace f32tc;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    if (*abort_flag && threadIdx.x == 0)
        tc::mbar_wait_bounded(reinterpret_cast<uint64_t *>(sm + kBar), phase, 1u << 22);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------------------
// sdf forward, tensor-core form with the coarse volumes in shared memory
// ---------------------------------------------------------------------------
// The point query of the tensor-core form (the gather, tile rows, product
// and epilogue of f32tc_decode, bit-identical results) as one persistent
// 16-warp block per SM.  The leading LODs whose volumes fit beside the tiles
// (5^3 and 9^3 vertices, 109 KB, at base_lod 2) are copied into shared
// memory once per block and gathered from there; only the finer LODs' corner
// lines come through L2.
//
// The block is four independent groups of four warps; group g decodes
// 128-point tiles g, g + 4, ... of the block's share into its own 128 TMEM
// columns (4 x 128 = the SM's 512).  A group gathers its tile in registers,
// takes one of two shared point-tile buffers, writes the split rows, and its
// first thread issues the tile's 14 MMAs; the group then gathers its next
// tile while the product runs, and only then reads the product back for the
// epilogue.  A buffer's lock covers its rows' stores and the issue; its
// next taker waits on the buffer's mbarrier for the product.  Groups meet
// only at their own named barrier (id 1 + g, 128 threads), never at a block
// barrier.
namespace f32st {
constexpr int kGroups = 4;
constexpr int kThreads = f32tc::kTP * kGroups;  // 512
constexpr int kStages = 2;                      // point-tile buffers
constexpr size_t kA = 0;                        // buffer b at kA + b f32tc::kTileA
constexpr size_t kW = (size_t)kStages * f32tc::kTileA;
constexpr size_t kW1 = kW + f32tc::kWBytes;
constexpr size_t kBar = kW1 + f32tc::kH * 4;    // one mbarrier per group: its product done
constexpr size_t kFree = kBar + 8 * kGroups;    // one mbarrier per buffer: its last product done
constexpr size_t kLock = kFree + 8 * kStages;   // int per buffer: 1 = taken
constexpr size_t kUses = kLock + 4 * kStages;   // uint32 per buffer: products issued on it
constexpr size_t kSel = kUses + 4 * kStages;    // int per group: its buffer, or -1
constexpr size_t kOk = kSel + 4 * kGroups;      // int per group: product done
constexpr size_t kSlot = kOk + 4 * kGroups;
constexpr size_t kAbort = kSlot + 4;
constexpr size_t kVol = (kAbort + 4 + 127) & ~(size_t)127;  // staged volumes
constexpr size_t kSmemMax = 227 * 1024;
constexpr size_t kVolBudget = kSmemMax - kVol;
// More than half of an SM's shared memory: one block per SM (its 512 TMEM
// columns are the SM's whole tensor memory).
constexpr size_t kSmemMin = 120 * 1024;
constexpr uint32_t kCols = kGroups * f32tc::kH;
static_assert(kW % 1024 == 0 && kBar % 8 == 0 && kFree % 8 == 0 && kVol % 128 == 0, "shared layout alignment");
static_assert(kVol + 109312 <= kSmemMax, "levels 5^3 and 9^3 fit");
}  // namespace f32st

__device__ __forceinline__ void group_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "n"(f32tc::kTP) : "memory");
}

// Takes a point-tile buffer whose last product has completed; -1 once the
// block is aborting, or (which also aborts it) if none came free within the
// bounds.  A buffer's lock covers only its rows' stores and the issue of its
// product; the next taker waits on the buffer's mbarrier for that product
// (uses: products issued on the buffer so far; the use before it completed
// before it was issued, so the barrier's parity is unambiguous).
__device__ __forceinline__ int acquire_tile_buffer(uint8_t *sm, uint32_t polls, volatile int *abort_flag) {
    using namespace f32st;
    int *locks = reinterpret_cast<int *>(sm + kLock);
    const uint32_t *uses = reinterpret_cast<const uint32_t *>(sm + kUses);
    for (uint32_t k = 0; k < (1u << 22); ++k) {
        if (*abort_flag) return -1;
#pragma unroll
        for (int b = 0; b < kStages; ++b)
            if (atomicCAS(&locks[b], 0, 1) == 0) {
                __threadfence_block();
                const uint32_t u = uses[b];
                if (u > 0 && !tc::mbar_wait_bounded(reinterpret_cast<uint64_t *>(sm + kFree) + b, (u - 1) & 1u, polls)) {
                    // the buffer's last product did not finish: the block
                    // stops (the buffer stays locked)
                    *abort_flag = 1;
                    atomicExch(&g_dense_status, 1);
                    return -1;
                }
                return b;
            }
        if (k > 16) __nanosleep(32);
    }
    *abort_flag = 1;
    atomicExch(&g_dense_status, 1);
    return -1;
}

__global__ void __launch_bounds__(f32st::kThreads, 1)
    sdf_fwd_f32_staged_kernel(const nglod_dense_model m, const float *__restrict__ x, int64_t n, int L, int staged,
                              float *__restrict__ out, uint32_t polls) {
    using namespace f32st;
    using f32tc::kH;
    using f32tc::kTileA;
    using f32tc::kTP;
    extern __shared__ __align__(1024) uint8_t smem_f32st[];
    uint8_t *sm = smem_f32st;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = warp >> 2, quad = warp & 3, gtid = tid & (kTP - 1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBar) + grp;
    uint64_t *freeb = reinterpret_cast<uint64_t *>(sm + kFree);
    int *locks = reinterpret_cast<int *>(sm + kLock);
    uint32_t *uses = reinterpret_cast<uint32_t *>(sm + kUses);
    volatile int *sel = reinterpret_cast<volatile int *>(sm + kSel) + grp;
    volatile int *okf = reinterpret_cast<volatile int *>(sm + kOk) + grp;
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + kSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kAbort);
    const float *sw1 = reinterpret_cast<const float *>(sm + kW1);

    // set-up: decoder, staged volumes, TMEM, barriers and locks
    stage_tf32_decoder(m, L, sm + kW, sm + kW1, tid, kThreads);
    {
        size_t off = kVol;
        for (int l = 0; l < staged; ++l) {
            const int s = volume_side(m, l);
            const int cnt = s * s * s * (kC / 4);
            const float4 *src = static_cast<const float4 *>(m.grid[l]);
            float4 *dst = reinterpret_cast<float4 *>(sm + off);
            for (int q = tid; q < cnt; q += kThreads) dst[q] = __ldg(src + q);
            off += (size_t)cnt * 16;
        }
    }
    if (warp == 0) tc::tmem_alloc(slot, kCols);
    if (tid == 0) {
        for (int g = 0; g < kGroups; ++g) tc::mbar_init(reinterpret_cast<uint64_t *>(sm + kBar) + g, 1);
        for (int b = 0; b < kStages; ++b) {
            tc::mbar_init(freeb + b, 1);
            locks[b] = 0;
            uses[b] = 0;
        }
        *abort_flag = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t sbase = tc::smem_addr(sm);
    const uint32_t dcol = tmem + (uint32_t)(grp * kH);
    const float b1 = m.b1[L][0];
    uint32_t phase = 0;
    bool pending = false;  // group leader: an issued product whose completion it did not see
    bool prev = false;     // the group has a tile whose epilogue is still to run
    int64_t prev_i = 0;    // that tile's point of this thread

    // Software-pipelined per group: the product of tile k runs while the
    // group gathers tile k + 1; then tile k's epilogue, then tile k + 1's
    // rows and product.
    const int64_t stride = (int64_t)gridDim.x * kGroups;
    // this thread's point of the group's next tile, loaded one tile ahead (the
    // points may be host memory read over the host link)
    float nx = 0.f, ny = 0.f, nz = 0.f;
    {
        const int64_t i0 = ((int64_t)blockIdx.x * kGroups + grp) * kTP + gtid;
        if (i0 < n) {
            nx = x[3 * i0];
            ny = x[3 * i0 + 1];
            nz = x[3 * i0 + 2];
        }
    }
    for (int64_t t = (int64_t)blockIdx.x * kGroups + grp;; t += stride) {
        const bool has = t * kTP < n;
        const int64_t i = t * kTP + gtid;
        const float px = nx, py = ny, pz = nz;
        {
            const int64_t in = i + stride * kTP;
            nx = ny = nz = 0.f;
            if (in < n) {
                nx = x[3 * in];
                ny = x[3 * in + 1];
                nz = x[3 * in + 2];
            }
        }
        float4 acc[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) acc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (has) {
            // 1. gather and LOD sum of the warp's 32 points (rows 32 quad ..)
            const float4 *vol = reinterpret_cast<const float4 *>(sm + kVol);
#pragma unroll 1
            for (int l = 0; l < staged; ++l) {
                const int s = volume_side(m, l);
                gather_warp_add_f32_shared(vol, s, px, py, pz, lane, acc);
                vol += s * s * s * (kC / 4);
            }
#pragma unroll 1
            for (int l = staged; l <= L; ++l)
                gather_warp_add_f32(static_cast<const float *>(m.grid[l]), volume_side(m, l), px, py, pz, lane, acc);
        }
        // 2. the previous tile's epilogue, once its product is done
        if (prev) {
            if (gtid == 0) {
                const bool ok = tc::mbar_wait_bounded(bar, phase, polls);
                if (ok) {
                    pending = false;
                } else {
                    *abort_flag = 1;
                    atomicExch(&g_dense_status, 1);
                }
                *okf = ok ? 1 : 0;
            }
            group_sync(grp);
            if (!*okf) break;
            phase ^= 1u;
            tc::fence_after_sync();
            const float o = relu_dot_w1_f32(dcol + ((uint32_t)(quad * 32) << 16), sw1);
            if (prev_i < n) out[prev_i] = o + b1;
            tc::fence_before_sync();
            prev = false;
        }
        if (!has) break;
        // 3. a point-tile buffer whose last product is done, the split rows
        if (gtid == 0) *sel = acquire_tile_buffer(sm, polls, abort_flag);
        group_sync(grp);
        const int b = *sel;
        if (b < 0) break;
        store_point_rows(sm + kA + (size_t)b * kTileA, quad * 32, lane, acc, px, py, pz);
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        group_sync(grp);
        // 4. the leader issues the tile's first layer; its completion arrives
        // on the group's barrier and on the buffer's, and the buffer's lock is
        // released at once
        if (gtid == 0) {
            tc::fence_after_sync();
            issue_first_layer(dcol, sbase + (uint32_t)(kA + b * kTileA), sbase + (uint32_t)kW);
            tc::mma_commit(bar);
            tc::mma_commit(freeb + b);
            pending = true;
            // A wait bound of 0 (nglod_debug_mma_wait_polls) cuts every wait
            // to one non-blocking test; the product is tested right after its
            // issue, where it is still running, so the error path runs.
            if (polls == 0 && !tc::mbar_test(bar, phase)) {
                *abort_flag = 1;
                atomicExch(&g_dense_status, 1);
            }
            uses[b] += 1;
            __threadfence_block();
            atomicExch(&locks[b], 0);
        }
        prev = true;
        prev_i = i;
    }
    // teardown: a product still in flight after a wait gave up finishes
    // before the columns are freed
    if (gtid == 0 && pending) tc::mbar_wait_bounded(bar, phase, 1u << 22);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// One feature volume sampled at every point: out[n][C] (FeatureVolume.forward).
// Cooperative gather (gather_warp_add_f32) of the warp's 32 points; each
// sample is written straight from the cooperative layout (four whole rows
// per store instruction).
__global__ void __launch_bounds__(256) volume_sample_f32_kernel(const float *__restrict__ g, int s,
                                                                const float *__restrict__ x, int64_t n,
                                                                float *__restrict__ out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
        gather_warp_add_f32(g, s, px, py, pz, lane, acc);
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int64_t ip = base + 4 * p + (lane >> 3);
            if (ip < n) reinterpret_cast<float4 *>(out + ip * kC)[lane & 7] = acc[p];
        }
    }
}

// ---------------------------------------------------------------------------
// ray vs [-1,1]^3 box
// ---------------------------------------------------------------------------

// Entry distance of a ray into the unit box, with the float arithmetic of
// sol_nglod_kernel.cu:92-150: reciprocal direction in double then float,
// slab distances (sgn - o) * invdir, entry-face tests with fmaf, the first
// passing face in x, y, z order, accepted when t < 500.  Rays starting inside
// the box return false.
__device__ __forceinline__ bool box_entry(float ox, float oy, float oz, float dx, float dy, float dz, float &t) {
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
    const float d = t0 ? d0 : (t1 ? d1 : (t2 ? d2 : 0.f));
    if ((t0 || t1 || t2) && d < 500.f) {
        t = d;
        return true;
    }
    return false;
}

__global__ void __launch_bounds__(256) aabb_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                                   int64_t n, float *__restrict__ x, float *__restrict__ t,
                                                   uint8_t *__restrict__ hit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float ox = ro[3 * i], oy = ro[3 * i + 1], oz = ro[3 * i + 2];
        const float dx = rd[3 * i], dy = rd[3 * i + 1], dz = rd[3 * i + 2];
        float tt = 0.f;
        const bool h = box_entry(ox, oy, oz, dx, dy, dz, tt);
        x[3 * i + 0] = h ? fmaf(dx, tt, ox) : ox;
        x[3 * i + 1] = h ? fmaf(dy, tt, oy) : oy;
        x[3 * i + 2] = h ? fmaf(dz, tt, oz) : oz;
        t[i] = h ? tt : 0.f;
        hit[i] = h ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------
// pinhole camera rays (look_at of sdf-net/lib/geoutils.py:180-206, no jitter)
// ---------------------------------------------------------------------------
struct CameraArgs {
    float eye[3], right[3], up[3], view[3];
    float tan_half;
    int width, height;
};

// Ray i = ix * height + iy (x-major, as torch.meshgrid(window_x, window_y)):
// pixel = right * wx * tan + up * wy * tan + eye + view with
// wx = (-1 + 2 ix / (W-1)) * W/H and wy = 1 - 2 iy / (H-1); origin = eye,
// direction = normalize(pixel - eye).
__global__ void camera_rays_kernel(const CameraArgs c, float *__restrict__ org, float *__restrict__ dir) {
    const int64_t n = (int64_t)c.width * c.height;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int ix = (int)(i / c.height), iy = (int)(i % c.height);
        const float wx = (c.width > 1 ? -1.f + 2.f * ix / (float)(c.width - 1) : 0.f) * ((float)c.width / c.height);
        const float wy = c.height > 1 ? 1.f - 2.f * iy / (float)(c.height - 1) : 0.f;
        float d[3];
        for (int k = 0; k < 3; ++k) d[k] = c.right[k] * wx * c.tan_half + c.up[k] * wy * c.tan_half + c.view[k];
        const float inv = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; ++k) {
            org[3 * i + k] = c.eye[k];
            dir[3 * i + k] = d[k] * inv;
        }
    }
}

// ---------------------------------------------------------------------------
// persistent sphere tracer
// ---------------------------------------------------------------------------
struct TraceArgs {
    nglod_dense_model m;
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
};

enum : int { kNeed = 0, kEvalInit = 1, kMarch = 2, kTap0 = 3, kDone = 9, kGone = 10 };

// One thread owns one ray at a time and every loop iteration evaluates exactly
// one sdf point per thread (the warp gathers its 32 points cooperatively): the ray's first point, its next march point, or
// one of the six finite-difference taps of its normal.  A thread whose ray
// finishes writes it out and takes the next ray index from a global counter;
// the lanes of a warp that need rays in the same iteration share one
// atomicAdd.  Per ray this runs SphereTracer.forward's state machine
// (SphereTracer.py:74-130): hit = |t| < far is re-evaluated at the start of
// every iteration, cond &= |d| > min_dis & |(d+dprev)/2| > osc_dis & hit,
// x = o + dir*t, dprev = d, d = net(x) * step_size, t += d; after the march
// hit &= all(|x| <= 1) and hit rays get normalize(central differences, h =
// 1/192).  Rays never affect one another in the reference, so running each to
// completion gives the same results as its global loop.
__global__ void __launch_bounds__(128) trace_f32_kernel(const TraceArgs a) {
    extern __shared__ float4 smem[];
    stage_decoder(smem, a.m, a.L);
    float *sT = reinterpret_cast<float *>(smem + decoder_f4(a.m.hidden_dim)) + (threadIdx.x >> 5) * 32 * kTRow;
    __syncthreads();

    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float h = 1.0f / 192.0f;
    const float twoh = (float)(2.0 / 192.0);

    int phase = kNeed, step = 0;
    int64_t ray = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f;
    float xx = 0.f, xy = 0.f, xz = 0.f, t = 0.f, d = 0.f, dprev = 0.f;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nx = 0.f, ny = 0.f, nz = 0.f;
    bool cond = false, hitr = false, hitf = false;

    auto finish = [&]() {
        hitf = hitr && !(fabsf(xx) > 1.f || fabsf(xy) > 1.f || fabsf(xz) > 1.f);
        phase = (hitf && a.p.want_normals) ? kTap0 : kDone;
    };
    // Start of march iteration `step` (SphereTracer.py:84-114).
    auto march_decide = [&]() {
        if (step >= a.p.num_steps) {
            finish();
            return;
        }
        hitr = fabsf(t) < a.p.far_clip;
        cond = cond && (fabsf(d) > a.p.min_dis) && (fabsf((d + dprev) / 2.f) > a.p.osc_dis) && hitr;
        if (!cond) {
            finish();
            return;
        }
        xx = __fadd_rn(ox, __fmul_rn(dx, t));
        xy = __fadd_rn(oy, __fmul_rn(dy, t));
        xz = __fadd_rn(oz, __fmul_rn(dz, t));
        dprev = d;
        phase = kMarch;
    };

    for (;;) {
        for (;;) {
            if (phase == kDone) {
                a.x[3 * ray + 0] = xx;
                a.x[3 * ray + 1] = xy;
                a.x[3 * ray + 2] = xz;
                a.t[ray] = t;
                a.hit[ray] = hitf ? 1 : 0;
                if (a.normal) {
                    const bool hn = hitf && a.p.want_normals;
                    a.normal[3 * ray + 0] = hn ? nx : 0.f;
                    a.normal[3 * ray + 1] = hn ? ny : 0.f;
                    a.normal[3 * ray + 2] = hn ? nz : 0.f;
                }
                phase = kNeed;
            }
            const unsigned need = __ballot_sync(FULL, phase == kNeed);
            if (need == 0u) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0ull;
            if ((int)lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (phase == kNeed) {
                const unsigned long long r = base + (unsigned long long)__popc(need & lt_mask);
                if (r >= (unsigned long long)a.n) {
                    phase = kGone;
                } else {
                    ray = (int64_t)r;
                    ox = a.ray_o[3 * ray];
                    oy = a.ray_o[3 * ray + 1];
                    oz = a.ray_o[3 * ray + 2];
                    dx = a.ray_d[3 * ray];
                    dy = a.ray_d[3 * ray + 1];
                    dz = a.ray_d[3 * ray + 2];
                    t = 0.f;
                    cond = box_entry(ox, oy, oz, dx, dy, dz, t);
                    xx = cond ? fmaf(dx, t, ox) : ox;
                    xy = cond ? fmaf(dy, t, oy) : oy;
                    xz = cond ? fmaf(dz, t, oz) : oz;
                    step = 0;
                    hitr = false;
                    hitf = false;
                    if (cond)
                        phase = kEvalInit;
                    else
                        march_decide();
                }
            }
        }
        if (__all_sync(FULL, phase == kGone)) break;

        float qx = xx, qy = xy, qz = xz;
        if (phase >= kTap0 && phase < kDone) {
            const int k = phase - kTap0;
            const float e = (k & 1) ? -h : h;
            if ((k >> 1) == 0) qx = __fadd_rn(xx, e);
            else if ((k >> 1) == 1) qy = __fadd_rn(xy, e);
            else qz = __fadd_rn(xz, e);
        }
        // every lane of the warp is here: the LOD sums of the warp's 32
        // points are gathered cooperatively, then each lane decodes its own
        float4 acc[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) acc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
        for (int l = 0; l <= a.L; ++l)
            gather_warp_add_f32(static_cast<const float *>(a.m.grid[l]), volume_side(a.m, l), qx, qy, qz, (int)lane,
                                acc);
        float f[kC];
        warp_sums_to_points(sT, (int)lane, acc, f);
        const float v = decode_f32(smem, a.m.hidden_dim, qx, qy, qz, f);

        if (phase == kEvalInit) {
            d = v;
            dprev = d;
            march_decide();
        } else if (phase == kMarch) {
            d = v * a.p.step_size;
            t = t + d;
            ++step;
            march_decide();
        } else if (phase >= kTap0 && phase < kDone) {
            const int k = phase - kTap0;
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
                phase = kDone;
            } else {
                phase = phase + 1;
            }
        }
    }
}

// The persistent float32 tracer with the tensor-core decode (hidden 128):
// trace_f32_kernel's state machine (SphereTracer.py:74-130) per thread, and
// every iteration the block's 256 query points (march points or normal taps)
// evaluated together by f32tc_decode, the float32 query kernel's arithmetic,
// so each evaluation gives the same bits as nglod_sdf_fwd at that point.
__global__ void __launch_bounds__(f32tc::kThreads, 2) trace_f32_tc_kernel(const TraceArgs a, uint32_t polls) {
    extern __shared__ __align__(1024) uint8_t smem_tr[];
    uint8_t *sm = smem_tr;
    const uint32_t tmem = f32tc_setup(a.m, a.L, sm, threadIdx.x);
    uint32_t mphase = 0;

    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float h = 1.0f / 192.0f;
    const float twoh = (float)(2.0 / 192.0);

    int phase = kNeed, step = 0;
    int64_t ray = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f;
    float xx = 0.f, xy = 0.f, xz = 0.f, t = 0.f, d = 0.f, dprev = 0.f;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nx = 0.f, ny = 0.f, nz = 0.f;
    bool cond = false, hitr = false, hitf = false;

    auto finish = [&]() {
        hitf = hitr && !(fabsf(xx) > 1.f || fabsf(xy) > 1.f || fabsf(xz) > 1.f);
        phase = (hitf && a.p.want_normals) ? kTap0 : kDone;
    };
    auto march_decide = [&]() {
        if (step >= a.p.num_steps) {
            finish();
            return;
        }
        hitr = fabsf(t) < a.p.far_clip;
        cond = cond && (fabsf(d) > a.p.min_dis) && (fabsf((d + dprev) / 2.f) > a.p.osc_dis) && hitr;
        if (!cond) {
            finish();
            return;
        }
        xx = __fadd_rn(ox, __fmul_rn(dx, t));
        xy = __fadd_rn(oy, __fmul_rn(dy, t));
        xz = __fadd_rn(oz, __fmul_rn(dz, t));
        dprev = d;
        phase = kMarch;
    };

    for (;;) {
        for (;;) {
            if (phase == kDone) {
                a.x[3 * ray + 0] = xx;
                a.x[3 * ray + 1] = xy;
                a.x[3 * ray + 2] = xz;
                a.t[ray] = t;
                a.hit[ray] = hitf ? 1 : 0;
                if (a.normal) {
                    const bool hn = hitf && a.p.want_normals;
                    a.normal[3 * ray + 0] = hn ? nx : 0.f;
                    a.normal[3 * ray + 1] = hn ? ny : 0.f;
                    a.normal[3 * ray + 2] = hn ? nz : 0.f;
                }
                phase = kNeed;
            }
            const unsigned need = __ballot_sync(FULL, phase == kNeed);
            if (need == 0u) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0ull;
            if ((int)lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (phase == kNeed) {
                const unsigned long long r = base + (unsigned long long)__popc(need & lt_mask);
                if (r >= (unsigned long long)a.n) {
                    phase = kGone;
                } else {
                    ray = (int64_t)r;
                    ox = a.ray_o[3 * ray];
                    oy = a.ray_o[3 * ray + 1];
                    oz = a.ray_o[3 * ray + 2];
                    dx = a.ray_d[3 * ray];
                    dy = a.ray_d[3 * ray + 1];
                    dz = a.ray_d[3 * ray + 2];
                    t = 0.f;
                    cond = box_entry(ox, oy, oz, dx, dy, dz, t);
                    xx = cond ? fmaf(dx, t, ox) : ox;
                    xy = cond ? fmaf(dy, t, oy) : oy;
                    xz = cond ? fmaf(dz, t, oz) : oz;
                    step = 0;
                    hitr = false;
                    hitf = false;
                    if (cond)
                        phase = kEvalInit;
                    else
                        march_decide();
                }
            }
        }
        if (__syncthreads_and(phase == kGone)) break;

        float qx = xx, qy = xy, qz = xz;
        if (phase >= kTap0 && phase < kDone) {
            const int k = phase - kTap0;
            const float e = (k & 1) ? -h : h;
            if ((k >> 1) == 0) qx = __fadd_rn(xx, e);
            else if ((k >> 1) == 1) qy = __fadd_rn(xy, e);
            else qz = __fadd_rn(xz, e);
        }
        if (phase == kGone) qx = qy = qz = 0.f;
        float v;
        if (!f32tc_decode(a.m, a.L, qx, qy, qz, sm, tmem, mphase, polls, v)) break;

        if (phase == kEvalInit) {
            d = v;
            dprev = d;
            march_decide();
        } else if (phase == kMarch) {
            d = v * a.p.step_size;
            t = t + d;
            ++step;
            march_decide();
        } else if (phase >= kTap0 && phase < kDone) {
            const int k = phase - kTap0;
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
                phase = kDone;
            } else {
                phase = phase + 1;
            }
        }
    }
    f32tc_teardown(sm, tmem, mphase);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
}  // namespace nglod

using namespace nglod;

extern "C" int nglod_aabb(const float *ray_o, const float *ray_d, int64_t n, float *x, float *t, uint8_t *hit,
                          nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && x && t && hit, NGLOD_ERR_INVALID, "null pointer argument");
    const int threads = 256;
    const int64_t want = (n + threads - 1) / threads;
    const int blocks = (int)(want < (int64_t)num_sms() * 16 ? want : (int64_t)num_sms() * 16);
    aabb_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(ray_o, ray_d, n, x, t, hit);
    return launch_status("nglod_aabb");
}

extern "C" int nglod_volume_sample(const float *grid, int32_t side, int32_t feature_dim, const float *x,
                                   int64_t n, float *out, nglod_stream_t stream) {
    NGLOD_REQUIRE(feature_dim == kC, NGLOD_ERR_UNSUPPORTED, "feature_dim=%d not built (only %d)", feature_dim, kC);
    NGLOD_REQUIRE(side >= 2 && side <= 1025, NGLOD_ERR_INVALID, "side=%d outside [2, 1025]", side);
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(grid && x && out, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(grid, 16) && aligned(out, 16), NGLOD_ERR_ALIGN, "grid and out must be 16-byte aligned");
    const int threads = 256;
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = resident_blocks(volume_sample_f32_kernel, threads, 0);
    volume_sample_f32_kernel<<<(int)(want < cap ? want : cap), threads, 0, (cudaStream_t)stream>>>(grid, side, x, n,
                                                                                                   out);
    return launch_status("nglod_volume_sample");
}

// The float32 query.  simt: the per-thread decoder (sdf_fwd_f32_kernel)
// even where the tensor-core form applies.
static int sdf_fwd_f32(const nglod_dense_model *model, const float *x, int64_t n, int32_t lod, int32_t all_lods,
                       float *out, cudaStream_t stream, bool simt) {
    NGLOD_REQUIRE(model != nullptr, NGLOD_ERR_INVALID, "model is null");
    const int L = all_lods ? model->num_lods - 1 : resolve_lod(model, lod);
    NGLOD_TRY(check_model(model, L));
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && out, NGLOD_ERR_INVALID, "null pointer argument");
    if (!all_lods && !simt && model->hidden_dim == f32tc::kH) {
        // the leading volumes that fit beside the tiles are staged
        int staged = 0;
        size_t vbytes = 0;
        for (int l = 0; l <= L; ++l) {
            const size_t s = (size_t)(1 << (l + model->base_lod)) + 1;
            if (vbytes + s * s * s * kC * 4 > f32st::kVolBudget) break;
            vbytes += s * s * s * kC * 4;
            ++staged;
        }
        const size_t smem = f32st::kVol + vbytes < f32st::kSmemMin ? f32st::kSmemMin : f32st::kVol + vbytes;
        auto k = sdf_fwd_f32_staged_kernel;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t tiles = (n + f32tc::kTP - 1) / f32tc::kTP;
        const int64_t want = (tiles + f32st::kGroups - 1) / f32st::kGroups;
        const int64_t cap = (int64_t)num_sms();
        k<<<(int)(want < cap ? want : cap), f32st::kThreads, smem, stream>>>(*model, x, n, L, staged, out,
                                                                           g_f32tc_wait_polls);
        return launch_status("nglod_sdf_fwd");
    }
    const int threads = 256;
    const int ndec = all_lods ? L + 1 : 1;
    // staged decoders, then one [32][kTRow] float transpose buffer per warp
    const size_t smem = (size_t)ndec * decoder_f4(model->hidden_dim) * sizeof(float4) +
                        (size_t)threads * kTRow * sizeof(float);
    const int64_t want = (n + threads - 1) / threads;
    if (all_lods) {
        auto k = sdf_fwd_f32_kernel<true>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, stream>>>(*model, x, n, L, out);
    } else {
        auto k = sdf_fwd_f32_kernel<false>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, stream>>>(*model, x, n, L, out);
    }
    return launch_status("nglod_sdf_fwd");
}

extern "C" int nglod_sdf_fwd(const nglod_dense_model *model, const float *x, int64_t n, int32_t lod,
                             int32_t all_lods, float *out, nglod_stream_t stream) {
    return sdf_fwd_f32(model, x, n, lod, all_lods, out, (cudaStream_t)stream, false);
}

extern "C" int nglod_sdf_fwd_simt(const nglod_dense_model *model, const float *x, int64_t n, int32_t lod,
                                  int32_t all_lods, float *out, nglod_stream_t stream) {
    return sdf_fwd_f32(model, x, n, lod, all_lods, out, (cudaStream_t)stream, true);
}

extern "C" int nglod_dense_status(int32_t *status_out) {
    NGLOD_REQUIRE(status_out != nullptr, NGLOD_ERR_INVALID, "null pointer argument");
    int32_t v = 0;
    const int32_t zero = 0;
    NGLOD_TRY(cuda_status(cudaMemcpyFromSymbol(&v, g_dense_status, sizeof(v)), "nglod_dense_status: read"));
    NGLOD_TRY(cuda_status(cudaMemcpyToSymbol(g_dense_status, &zero, sizeof(zero)), "nglod_dense_status: reset"));
    *status_out = v;
    return NGLOD_OK;
}

void nglod::set_f32tc_wait_polls(uint32_t polls) { g_f32tc_wait_polls = polls; }

namespace {
struct F32HostCtx {
    const nglod_dense_model *model;
    int32_t lod;
};
int f32_host_chunk(const void *ctx, const float *x, int64_t m, float *out, cudaStream_t s) {
    const F32HostCtx *c = static_cast<const F32HostCtx *>(ctx);
    return nglod_sdf_fwd(c->model, x, m, c->lod, 0, out, (nglod_stream_t)s);
}
}  // namespace

extern "C" int nglod_sdf_fwd_host(const nglod_dense_model *model, const float *x_host, int64_t n, int32_t lod,
                                  float *out_host, int64_t chunk, void *scratch, nglod_stream_t stream) {
    NGLOD_TRY(nglod_sdf_fwd(model, nullptr, 0, lod, 0, nullptr, stream));  // validates the model
    const F32HostCtx ctx{model, lod};
    return host_query_pipeline(x_host, n, out_host, chunk, scratch, (cudaStream_t)stream, f32_host_chunk, &ctx);
}

extern "C" int nglod_trace(const nglod_dense_model *model, const nglod_trace_params *params, const float *ray_o,
                           const float *ray_d, int64_t n, float *x, float *t, uint8_t *hit, float *normal,
                           int64_t *work_counter, nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr && params != nullptr, NGLOD_ERR_INVALID, "model or params is null");
    const int L = resolve_lod(model, params->lod);
    NGLOD_TRY(check_model(model, L));
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    NGLOD_REQUIRE(params->num_steps >= 0, NGLOD_ERR_INVALID, "num_steps=%d is negative", params->num_steps);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && x && t && hit && work_counter, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(normal || !params->want_normals, NGLOD_ERR_INVALID, "normals requested with a null buffer");
    NGLOD_REQUIRE(aligned(work_counter, 8), NGLOD_ERR_ALIGN, "work_counter is not 8-byte aligned");
    TraceArgs a;
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
    NGLOD_TRY(cuda_status(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), (cudaStream_t)stream),
                          "nglod_trace counter reset"));
    if (model->hidden_dim == f32tc::kH) {
        // tensor-core decode, 256 rays per block, two blocks per SM
        NGLOD_TRY(prepare_smem(trace_f32_tc_kernel, f32tc::kSmem));
        const int64_t want = (n + f32tc::kThreads - 1) / f32tc::kThreads;
        const int64_t cap = (int64_t)num_sms() * 2;
        trace_f32_tc_kernel<<<(int)(want < cap ? want : cap), f32tc::kThreads, f32tc::kSmem, (cudaStream_t)stream>>>(
            a, g_f32tc_wait_polls);
        return launch_status("nglod_trace");
    }
    const int threads = 128;
    // staged decoder, then one [32][kTRow] float transpose buffer per warp
    const size_t smem = (size_t)decoder_f4(model->hidden_dim) * sizeof(float4) + (size_t)threads * kTRow * sizeof(float);
    NGLOD_TRY(prepare_smem(trace_f32_kernel, smem));
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = resident_blocks(trace_f32_kernel, threads, smem);
    trace_f32_kernel<<<(int)(want < cap ? want : cap), threads, smem, (cudaStream_t)stream>>>(a);
    return launch_status("nglod_trace");
}

extern "C" int nglod_camera_rays(const float *eye, const float *at, const float *up, float fov_deg, int32_t width,
                                 int32_t height, float *org, float *dir, nglod_stream_t stream) {
    NGLOD_REQUIRE(eye && at && up && org && dir, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(width > 0 && height > 0, NGLOD_ERR_INVALID, "image %dx%d is empty", width, height);
    CameraArgs c;
    double v[3], r[3], u[3], nv = 0, nr = 0, nu = 0;
    for (int k = 0; k < 3; ++k) {
        v[k] = (double)at[k] - eye[k];
        nv += v[k] * v[k];
    }
    nv = sqrt(nv);
    NGLOD_REQUIRE(nv > 0, NGLOD_ERR_INVALID, "eye and target coincide");
    for (int k = 0; k < 3; ++k) v[k] /= nv;
    r[0] = v[1] * up[2] - v[2] * up[1];
    r[1] = v[2] * up[0] - v[0] * up[2];
    r[2] = v[0] * up[1] - v[1] * up[0];
    for (int k = 0; k < 3; ++k) nr += r[k] * r[k];
    nr = sqrt(nr);
    NGLOD_REQUIRE(nr > 0, NGLOD_ERR_INVALID, "up is parallel to the view direction");
    for (int k = 0; k < 3; ++k) r[k] /= nr;
    u[0] = r[1] * v[2] - r[2] * v[1];
    u[1] = r[2] * v[0] - r[0] * v[2];
    u[2] = r[0] * v[1] - r[1] * v[0];
    for (int k = 0; k < 3; ++k) nu += u[k] * u[k];
    nu = sqrt(nu);
    for (int k = 0; k < 3; ++k) {
        c.eye[k] = eye[k];
        c.view[k] = (float)v[k];
        c.right[k] = (float)r[k];
        c.up[k] = (float)(u[k] / nu);
    }
    c.tan_half = (float)tan(fov_deg * 3.14159265358979323846 / 360.0);
    c.width = width;
    c.height = height;
    const int64_t n = (int64_t)width * height;
    const int64_t want = (n + 255) / 256, cap = (int64_t)num_sms() * 16;
    camera_rays_kernel<<<(int)(want < cap ? want : cap), 256, 0, (cudaStream_t)stream>>>(c, org, dir);
    return launch_status("nglod_camera_rays");
}
