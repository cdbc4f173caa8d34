// Sparse SDF on an SPC octree: corner-feature / trinket construction, point
// queries and a persistent sparse sphere tracer (sol-renderer's SDF class).
//
// Feature lookup for a point in voxel g of level lod+2 walks g and its
// parents down to level 2; at each level the 8 corner features of the voxel
// (corner_idx[g]) are blended with trilinear weights computed from the
// voxel's own integer coordinates, which are the corner coordinates the
// reference reads from its cc table (solr/sdf/sparse_grid_sample.cuh:52-107).
// The tensor-core tracer can read the corner indices of every level from a
// per-voxel chain row instead (corner_chain), so no load waits on a parent
// index.
#include <vector>

#include "bf16_tile.cuh"
#include "dense_common.cuh"
#include "scan.cuh"

namespace nglod {

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

// Adds the 32 features of corner row `k`, scaled by w, to f.
template <int DT>
__device__ __forceinline__ void add_corner(const void *feats, int64_t k, float w, float (&f)[kC]) {
    if (DT == NGLOD_F32) {
        const float4 *r = reinterpret_cast<const float4 *>(feats) + k * (kC / 4);
#pragma unroll
        for (int q = 0; q < kC / 4; ++q) {
            const float4 v = __ldg(r + q);
            f[4 * q] = fmaf(v.x, w, f[4 * q]);
            f[4 * q + 1] = fmaf(v.y, w, f[4 * q + 1]);
            f[4 * q + 2] = fmaf(v.z, w, f[4 * q + 2]);
            f[4 * q + 3] = fmaf(v.w, w, f[4 * q + 3]);
        }
    } else {
        const uint4 *r = reinterpret_cast<const uint4 *>(feats) + k * (kC / 8);
#pragma unroll
        for (int q = 0; q < kC / 8; ++q) {
            const uint4 v = __ldg(r + q);
            f[8 * q + 0] = fmaf(bf16_lo(v.x), w, f[8 * q + 0]);
            f[8 * q + 1] = fmaf(bf16_hi(v.x), w, f[8 * q + 1]);
            f[8 * q + 2] = fmaf(bf16_lo(v.y), w, f[8 * q + 2]);
            f[8 * q + 3] = fmaf(bf16_hi(v.y), w, f[8 * q + 3]);
            f[8 * q + 4] = fmaf(bf16_lo(v.z), w, f[8 * q + 4]);
            f[8 * q + 5] = fmaf(bf16_hi(v.z), w, f[8 * q + 5]);
            f[8 * q + 6] = fmaf(bf16_lo(v.w), w, f[8 * q + 6]);
            f[8 * q + 7] = fmaf(bf16_hi(v.w), w, f[8 * q + 7]);
        }
    }
}

// Sum over levels lod+2 .. 2 of the trilinear corner blend at p, starting in
// voxel g (global point index at level lod+2).  Corners are visited x
// fastest, then y, then z, as the reference accumulates them; the position
// is normalised with fmaf(x, 0.5, 0.5) and scaled by 2^level.
template <int DT>
__device__ __forceinline__ void sparse_features(const nglod_sparse_model &m, int lod, int64_t g, float px, float py,
                                                float pz, float (&f)[kC]) {
#pragma unroll
    for (int c = 0; c < kC; ++c) f[c] = 0.f;
    const float nx = fmaf(px, 0.5f, 0.5f), ny = fmaf(py, 0.5f, 0.5f), nz = fmaf(pz, 0.5f, 0.5f);
    const int last = m.summed ? lod + 2 : 2;  // LOD-summed features: the query level alone
#pragma unroll 1
    for (int lv = lod + 2; lv >= last; --lv) {
        if (lv != lod + 2) g = m.parent[g];
        const float res = (float)(1 << lv);
        const float ux = nx * res, uy = ny * res, uz = nz * res;
        const short4 p = reinterpret_cast<const short4 *>(m.points)[g];
        const float x0 = (float)p.x, y0 = (float)p.y, z0 = (float)p.z;
        const float wx[2] = {(x0 + 1.f) - ux, ux - x0};
        const float wy[2] = {(y0 + 1.f) - uy, uy - y0};
        const float wz[2] = {(z0 + 1.f) - uz, uz - z0};
        const int4 ca = __ldg(reinterpret_cast<const int4 *>(m.corner_idx) + 2 * g);
        const int4 cb = __ldg(reinterpret_cast<const int4 *>(m.corner_idx) + 2 * g + 1);
        const int ci[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int bx = k & 1, by = (k >> 1) & 1, bz = k >> 2;
            const float w = (wz[bz] * wy[by]) * wx[bx];
            add_corner<DT>(m.corner_feats, ci[4 * bx + 2 * by + bz], w, f);
        }
    }
}

// ---------------------------------------------------------------------------
// voxel entry (solr/gfx/ray_aabb.cuh:42-89)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float voxel_entry(float qx, float qy, float qz, float dx, float dy, float dz, float ivx,
                                             float ivy, float ivz, float sx, float sy, float sz, float cx, float cy,
                                             float cz, float r) {
    const float ox = qx - cx, oy = qy - cy, oz = qz - cz;
    const float cmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
    float winding = cmax < r ? -1.f : 1.f;
    winding *= r;
    if (winding < 0.f) return winding;
    const float d0 = __fmul_rn(__fmaf_rn(winding, sx, -ox), ivx);
    const float d1 = __fmul_rn(__fmaf_rn(winding, sy, -oy), ivy);
    const float d2 = __fmul_rn(__fmaf_rn(winding, sz, -oz), ivz);
    const bool t0 = (d0 >= 0.f) && (fabsf(__fmaf_rn(dy, d0, oy)) < r) && (fabsf(__fmaf_rn(dz, d0, oz)) < r);
    const bool t1 = (d1 >= 0.f) && (fabsf(__fmaf_rn(dx, d1, ox)) < r) && (fabsf(__fmaf_rn(dz, d1, oz)) < r);
    const bool t2 = (d2 >= 0.f) && (fabsf(__fmaf_rn(dx, d2, ox)) < r) && (fabsf(__fmaf_rn(dy, d2, oy)) < r);
    return t0 ? d0 : (t1 ? d1 : (t2 ? d2 : 0.f));
}

// ---------------------------------------------------------------------------
// persistent sparse tracer
// ---------------------------------------------------------------------------
struct SparseTraceArgs {
    nglod_sparse_model m;
    int lod;
    int num_steps;
    const float *ray_o;
    const float *ray_d;
    int64_t n;
    const int2 *nug;
    int64_t n_nug;
    const int32_t *ray_first;
    float *x;
    float *t;
    uint8_t *hit;
    float *normal;
    unsigned long long *counter;
};

__global__ void ray_first_kernel(const int2 *__restrict__ nug, int64_t m, int32_t *__restrict__ first) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
        if (i == 0 || nug[i - 1].x != nug[i].x) first[nug[i].x] = (int32_t)i;
}

enum : int { sNeed = 0, sMarch = 1, sTap0 = 2, sDone = 8, sGone = 9 };

template <int DT>
__global__ void __launch_bounds__(128) sparse_trace_kernel(const SparseTraceArgs a) {
    extern __shared__ float4 smem[];
    const int H = a.m.hidden_dim;
    stage_decoder_ptrs(smem, H, a.m.w0[a.lod], a.m.b0[a.lod], a.m.w1[a.lod], a.m.b1[a.lod]);
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int level = a.lod + 2;
    const int64_t lstart = a.m.level_start[level];
    const float r = (float)(1.0 / (double)(1 << level));
    const float eps = 0.001f;

    int phase = sNeed, it = 0;
    int64_t ray = 0, pidx = 0;
    int first = -1;
    float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f, ivx = 0.f, ivy = 0.f, ivz = 0.f;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float xx = 0.f, xy = 0.f, xz = 0.f, t = 0.f, dprev = 0.f;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nx = 1.f, ny = 1.f, nz = 1.f;
    bool cond = false, hitf = false;

    // First voxel along the ray's nugget list that contains or lies ahead of
    // (qx, qy, qz); ray_aabb_kernel (ray_aabb.cuh:104-192).
    auto walk = [&](float qx, float qy, float qz) {
        bool found = false;
        int64_t i = first;
        do {
            const int pid = a.nug[i].y;
            const short4 p = reinterpret_cast<const short4 *>(a.m.points)[lstart + pid];
            const float cx = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.x, 1.f), -1.f);
            const float cy = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.y, 1.f), -1.f);
            const float cz = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.z, 1.f), -1.f);
            const float dd = voxel_entry(qx, qy, qz, dx, dy, dz, ivx, ivy, ivz, sx, sy, sz, cx, cy, cz, r);
            if (dd != 0.f) {
                found = true;
                pidx = lstart + pid;
                cond = true;
                if (dd > 0.f) {
                    t = t + dd;
                    xx = __fmaf_rn(dx, t, ox);
                    xy = __fmaf_rn(dy, t, oy);
                    xz = __fmaf_rn(dz, t, oz);
                }
            }
            ++i;
        } while (i < a.n_nug && a.nug[i].x == (int)ray && !found);
        if (!found) {
            cond = false;
            t = 100.f;
            xx = __fmaf_rn(dx, t, ox);
            xy = __fmaf_rn(dy, t, oy);
            xz = __fmaf_rn(dz, t, oz);
        }
    };

    for (;;) {
        for (;;) {
            if (phase == sDone) {
                a.x[3 * ray + 0] = xx;
                a.x[3 * ray + 1] = xy;
                a.x[3 * ray + 2] = xz;
                a.t[ray] = t;
                a.hit[ray] = hitf ? 1 : 0;
                if (a.normal) {
                    a.normal[3 * ray + 0] = hitf ? nx : 1.f;
                    a.normal[3 * ray + 1] = hitf ? ny : 1.f;
                    a.normal[3 * ray + 2] = hitf ? nz : 1.f;
                }
                phase = sNeed;
            }
            const unsigned need = __ballot_sync(FULL, phase == sNeed);
            if (need == 0u) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0ull;
            if ((int)lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (phase == sNeed) {
                const unsigned long long rr = base + (unsigned long long)__popc(need & lt_mask);
                if (rr >= (unsigned long long)a.n) {
                    phase = sGone;
                    continue;
                }
                ray = (int64_t)rr;
                ox = a.ray_o[3 * ray];
                oy = a.ray_o[3 * ray + 1];
                oz = a.ray_o[3 * ray + 2];
                dx = a.ray_d[3 * ray];
                dy = a.ray_d[3 * ray + 1];
                dz = a.ray_d[3 * ray + 2];
                xx = ox;
                xy = oy;
                xz = oz;
                t = 0.f;
                dprev = 0.f;
                it = 0;
                cond = false;
                hitf = false;
                first = a.ray_first[ray];
                if (first < 0) {
                    phase = sDone;
                    continue;
                }
                ivx = __fdiv_rn(1.f, dx);
                ivy = __fdiv_rn(1.f, dy);
                ivz = __fdiv_rn(1.f, dz);
                sx = signbit(dx) ? 1.f : -1.f;
                sy = signbit(dy) ? 1.f : -1.f;
                sz = signbit(dz) ? 1.f : -1.f;
                walk(ox, oy, oz);
                phase = (cond && a.num_steps > 0) ? sMarch : sDone;
            }
        }
        if (__all_sync(FULL, phase == sGone)) break;

        float qx = xx, qy = xy, qz = xz;
        if (phase >= sTap0 && phase < sDone) {
            const int k = phase - sTap0;
            const float e = (k & 1) ? -eps : eps;
            if ((k >> 1) == 0) qx = __fadd_rn(xx, e);
            else if ((k >> 1) == 1) qy = __fadd_rn(xy, e);
            else qz = __fadd_rn(xz, e);
        }
        float f[kC];
        sparse_features<DT>(a.m, a.lod, phase == sGone ? lstart : pidx, qx, qy, qz, f);
        const float v = decode_f32(smem, H, qx, qy, qz, f);

        if (phase == sMarch) {
            // step_kernel (solr/sdf/step.cuh:48-85); thresholds compared in double
            const float d = v;
            t = t + d;
            hitf = ((double)fabsf(d) < 0.0003) || ((double)fabsf(d + dprev) * 0.5 < 0.0015);
            cond = ((double)t < 5.0) && !hitf;
            xx = __fmaf_rn(dx, t, ox);
            xy = __fmaf_rn(dy, t, oy);
            xz = __fmaf_rn(dz, t, oz);
            dprev = d;
            ++it;
            if (cond) walk(xx, xy, xz);
            if (!cond || it >= a.num_steps) phase = hitf ? sTap0 : sDone;
        } else if (phase >= sTap0 && phase < sDone) {
            const int k = phase - sTap0;
#pragma unroll
            for (int i = 0; i < 6; ++i)
                if (i == k) g[i] = v;
            if (k == 5) {
                const float gx = g[0] - g[1], gy = g[2] - g[3], gz = g[4] - g[5];
                const float nrm = norm3df(gx, gy, gz);
                nx = gx / nrm;
                ny = gy / nrm;
                nz = gz / nrm;
                phase = sDone;
            } else {
                phase = phase + 1;
            }
        }
    }
}

// corner_chain rows of the level-(lod+2) voxels start .. start+count-1: row
// v, block k = corner_idx of the voxel k parent steps above voxel start+v.
__global__ void chain_build_kernel(const int4 *__restrict__ corner_idx, const int32_t *__restrict__ parent,
                                   int64_t start, int64_t count, int lod, int4 *__restrict__ chain) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < count; v += stride) {
        int64_t g = start + v;
        int4 *row = chain + v * (lod + 1) * 2;
        for (int k = 0; k <= lod; ++k) {
            if (k > 0) g = parent[g];
            row[2 * k] = corner_idx[2 * g];
            row[2 * k + 1] = corner_idx[2 * g + 1];
        }
    }
}

// ---------------------------------------------------------------------------
// persistent sparse tracer with the BF16 tensor-core decoder
// ---------------------------------------------------------------------------
// This lane's 8 channels (8q .. 8q+7) of sparse_features<NGLOD_BF16>: the
// same corners, weights and per-channel fmaf order.  kChain: the corner
// indices of every level come from the voxel's own corner_chain row and the
// ancestors' coordinates are the voxel's shifted right (an octree parent is
// the voxel at half the coordinates), so no load waits on a parent index.
template <bool kChain>
__device__ __forceinline__ void sparse_features_quarter(const nglod_sparse_model &m, int lod, int64_t g, float px,
                                                        float py, float pz, int q, float (&f)[8]) {
    // channel pairs (2c, 2c + 1) in one packed FMA: each lane of it is the
    // same float32 FMA as before, in the same corner order
    float2 f2[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) f2[c] = make_float2(0.f, 0.f);
    const float nx = fmaf(px, 0.5f, 0.5f), ny = fmaf(py, 0.5f, 0.5f), nz = fmaf(pz, 0.5f, 0.5f);
    const uint4 *feats = static_cast<const uint4 *>(m.corner_feats) + q;  // 4 uint4 per corner row
    const short4 pf = reinterpret_cast<const short4 *>(m.points)[g];
    const int4 *chain =
        kChain ? reinterpret_cast<const int4 *>(m.corner_chain[lod]) + (g - m.level_start[lod + 2]) * (lod + 1) * 2
               : nullptr;
    // kChain: the next level's corner indices are loaded one level ahead
    int4 na = make_int4(0, 0, 0, 0), nb = na;
    if (kChain) {
        na = __ldg(chain);
        nb = __ldg(chain + 1);
    }
    const int last = m.summed ? lod + 2 : 2;  // LOD-summed features: the query level alone
#pragma unroll 1
    for (int lv = lod + 2; lv >= last; --lv) {
        const int k = lod + 2 - lv;
        short4 p;
        int4 ca, cb;
        if (kChain) {
            p = make_short4((short)(pf.x >> k), (short)(pf.y >> k), (short)(pf.z >> k), 0);
            ca = na;
            cb = nb;
            if (k < lod && !m.summed) {
                na = __ldg(chain + 2 * k + 2);
                nb = __ldg(chain + 2 * k + 3);
            }
        } else {
            if (lv != lod + 2) g = m.parent[g];
            p = lv == lod + 2 ? pf : reinterpret_cast<const short4 *>(m.points)[g];
            ca = __ldg(reinterpret_cast<const int4 *>(m.corner_idx) + 2 * g);
            cb = __ldg(reinterpret_cast<const int4 *>(m.corner_idx) + 2 * g + 1);
        }
        const float res = (float)(1 << lv);
        const float ux = nx * res, uy = ny * res, uz = nz * res;
        const float x0 = (float)p.x, y0 = (float)p.y, z0 = (float)p.z;
        const float wx[2] = {(x0 + 1.f) - ux, ux - x0};
        const float wy[2] = {(y0 + 1.f) - uy, uy - y0};
        const float wz[2] = {(z0 + 1.f) - uz, uz - z0};
        const int ci[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
        uint4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int bx = k & 1, by = (k >> 1) & 1, bz = k >> 2;
            v[k] = __ldg(feats + (int64_t)ci[4 * bx + 2 * by + bz] * 4);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int bx = k & 1, by = (k >> 1) & 1, bz = k >> 2;
            const float w = (wz[bz] * wy[by]) * wx[bx];
            const float2 w2 = make_float2(w, w);
            f2[0] = __ffma2_rn(make_float2(bf16_lo(v[k].x), bf16_hi(v[k].x)), w2, f2[0]);
            f2[1] = __ffma2_rn(make_float2(bf16_lo(v[k].y), bf16_hi(v[k].y)), w2, f2[1]);
            f2[2] = __ffma2_rn(make_float2(bf16_lo(v[k].z), bf16_hi(v[k].z)), w2, f2[2]);
            f2[3] = __ffma2_rn(make_float2(bf16_lo(v[k].w), bf16_hi(v[k].w)), w2, f2[3]);
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        f[2 * c] = f2[c].x;
        f[2 * c + 1] = f2[c].y;
    }
}

struct SparseTcArgs {
    SparseTraceArgs t;
    int *status;
};

// The state machine of sparse_trace_kernel (step_kernel rules, nugget walk,
// getNormal taps) with every sdf evaluation done for 128 rays at once: each
// slot publishes its query point and voxel, the block gathers the 128 rows'
// corner features into the bf16 tile, one thread issues the tcgen05 product
// and each thread reads its row's hidden layer back for the fp32 epilogue.
template <bool kChain>
__global__ void __launch_bounds__(kTP, 4) sparse_trace_tc_kernel(const SparseTcArgs args) {
    const SparseTraceArgs &a = args.t;
    // the block's dynamic shared memory, as bytes (the float32 kernels of this
    // file declare it as float4)
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    uint8_t *sA = smem_tc + kSmemA;
    uint8_t *sB = smem_tc + kSmemB;
    float *sw1 = reinterpret_cast<float *>(smem_tc + kSmemW1);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_tc + kSmemBar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem_tc + kSmemSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem_tc + kSmemAbort);
    float4 *qpts = reinterpret_cast<float4 *>(smem_tc + kSmemQ);

    const int tid = threadIdx.x, warp = tid >> 5;
    const unsigned lane = threadIdx.x & 31u;
    const uint4 *bsrc = static_cast<const uint4 *>(a.m.w0_tile[a.lod]);
    for (int i = tid; i < (int)(kTileBytes / 16); i += kTP) reinterpret_cast<uint4 *>(sB)[i] = bsrc[i];
    sw1[tid] = a.m.w1[a.lod][tid];
    const float b1 = a.m.b1[a.lod][0];
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

    const unsigned FULL = 0xffffffffu;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int level = a.lod + 2;
    const int64_t lstart = a.m.level_start[level];
    const float r = (float)(1.0 / (double)(1 << level));
    const float eps = 0.001f;

    int phase = sNeed, it = 0;
    int64_t ray = 0, pidx = 0;
    int first = -1;
    float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f, ivx = 0.f, ivy = 0.f, ivz = 0.f;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float xx = 0.f, xy = 0.f, xz = 0.f, t = 0.f, dprev = 0.f;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nx = 1.f, ny = 1.f, nz = 1.f;
    bool cond = false, hitf = false;

    auto walk = [&](float qx, float qy, float qz) {
        bool found = false;
        int64_t i = first;
        do {
            const int pid = a.nug[i].y;
            const short4 p = reinterpret_cast<const short4 *>(a.m.points)[lstart + pid];
            const float cx = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.x, 1.f), -1.f);
            const float cy = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.y, 1.f), -1.f);
            const float cz = __fmaf_rn(r, __fmaf_rn(2.f, (float)p.z, 1.f), -1.f);
            const float dd = voxel_entry(qx, qy, qz, dx, dy, dz, ivx, ivy, ivz, sx, sy, sz, cx, cy, cz, r);
            if (dd != 0.f) {
                found = true;
                pidx = lstart + pid;
                cond = true;
                if (dd > 0.f) {
                    t = t + dd;
                    xx = __fmaf_rn(dx, t, ox);
                    xy = __fmaf_rn(dy, t, oy);
                    xz = __fmaf_rn(dz, t, oz);
                }
            }
            ++i;
        } while (i < a.n_nug && a.nug[i].x == (int)ray && !found);
        if (!found) {
            cond = false;
            t = 100.f;
            xx = __fmaf_rn(dx, t, ox);
            xy = __fmaf_rn(dy, t, oy);
            xz = __fmaf_rn(dz, t, oz);
        }
    };

    for (;;) {
        for (;;) {
            if (phase == sDone) {
                a.x[3 * ray + 0] = xx;
                a.x[3 * ray + 1] = xy;
                a.x[3 * ray + 2] = xz;
                a.t[ray] = t;
                a.hit[ray] = hitf ? 1 : 0;
                if (a.normal) {
                    a.normal[3 * ray + 0] = hitf ? nx : 1.f;
                    a.normal[3 * ray + 1] = hitf ? ny : 1.f;
                    a.normal[3 * ray + 2] = hitf ? nz : 1.f;
                }
                phase = sNeed;
            }
            const unsigned need = __ballot_sync(FULL, phase == sNeed);
            if (need == 0u) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0ull;
            if ((int)lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (phase == sNeed) {
                const unsigned long long rr = base + (unsigned long long)__popc(need & lt_mask);
                if (rr >= (unsigned long long)a.n) {
                    phase = sGone;
                    continue;
                }
                ray = (int64_t)rr;
                ox = a.ray_o[3 * ray];
                oy = a.ray_o[3 * ray + 1];
                oz = a.ray_o[3 * ray + 2];
                dx = a.ray_d[3 * ray];
                dy = a.ray_d[3 * ray + 1];
                dz = a.ray_d[3 * ray + 2];
                xx = ox;
                xy = oy;
                xz = oz;
                t = 0.f;
                dprev = 0.f;
                it = 0;
                cond = false;
                hitf = false;
                first = a.ray_first[ray];
                if (first < 0) {
                    phase = sDone;
                    continue;
                }
                ivx = __fdiv_rn(1.f, dx);
                ivy = __fdiv_rn(1.f, dy);
                ivz = __fdiv_rn(1.f, dz);
                sx = signbit(dx) ? 1.f : -1.f;
                sy = signbit(dy) ? 1.f : -1.f;
                sz = signbit(dz) ? 1.f : -1.f;
                walk(ox, oy, oz);
                phase = (cond && a.num_steps > 0) ? sMarch : sDone;
            }
        }
        if (__syncthreads_and(phase == sGone)) break;

        float qx = xx, qy = xy, qz = xz;
        if (phase >= sTap0 && phase < sDone) {
            const int k = phase - sTap0;
            const float e = (k & 1) ? -eps : eps;
            if ((k >> 1) == 0) qx = __fadd_rn(xx, e);
            else if ((k >> 1) == 1) qy = __fadd_rn(xy, e);
            else qz = __fadd_rn(xz, e);
        }
        if (phase == sGone) qx = qy = qz = 0.f;
        qpts[tid] = make_float4(qx, qy, qz, __int_as_float((int)(phase == sGone ? lstart : pidx)));
        __syncthreads();
        // gather: warp w fills rows 32w .. 32w+31, eight points per pass
#pragma unroll 1
        for (int pass = 0; pass < 4; ++pass) {
            const int row = warp * 32 + pass * 8 + (int)(lane >> 2), q = (int)(lane & 3u);
            const float4 pt = qpts[row];
            float f[8];
            sparse_features_quarter<kChain>(a.m, a.lod, (int64_t)__float_as_int(pt.w), pt.x, pt.y, pt.z, q, f);
            *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, 8 * q)) =
                make_uint4(pack_bf16x2(f[0], f[1]), pack_bf16x2(f[2], f[3]), pack_bf16x2(f[4], f[5]),
                           pack_bf16x2(f[6], f[7]));
            if (q == 0)
                *reinterpret_cast<uint4 *>(sA + tile_offset_a(row, 32)) = position_columns(pt.x, pt.y, pt.z);
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
                atomicExch(args.status, 1);
            }
        }
        __syncthreads();
        if (*abort_flag) break;
        mphase ^= 1u;
        tc::fence_after_sync();
        const float v = relu_dot_w1(tmem + ((uint32_t)(warp * 32) << 16), sw1) + b1;
        tc::fence_before_sync();

        if (phase == sMarch) {
            // step_kernel (solr/sdf/step.cuh:48-85); thresholds compared in double
            const float d = v;
            t = t + d;
            hitf = ((double)fabsf(d) < 0.0003) || ((double)fabsf(d + dprev) * 0.5 < 0.0015);
            cond = ((double)t < 5.0) && !hitf;
            xx = __fmaf_rn(dx, t, ox);
            xy = __fmaf_rn(dy, t, oy);
            xz = __fmaf_rn(dz, t, oz);
            dprev = d;
            ++it;
            if (cond) walk(xx, xy, xz);
            if (!cond || it >= a.num_steps) phase = hitf ? sTap0 : sDone;
        } else if (phase >= sTap0 && phase < sDone) {
            const int k = phase - sTap0;
#pragma unroll
            for (int i = 0; i < 6; ++i)
                if (i == k) g[i] = v;
            if (k == 5) {
                const float gx = g[0] - g[1], gy = g[2] - g[3], gz = g[4] - g[5];
                const float nrm = norm3df(gx, gy, gz);
                nx = gx / nrm;
                ny = gy / nrm;
                nz = gz / nrm;
                phase = sDone;
            } else {
                phase = phase + 1;
            }
        }
        // the next iteration's gather overwrites the A tile only after every
        // thread has read its TMEM row (the __syncthreads_and above)
    }
    if (*abort_flag && tid == 0) tc::mbar_wait_bounded(bar, mphase, kWaitPolls);  // let an in-flight MMA finish
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kHid);
}

// ---------------------------------------------------------------------------
// point query (SDF::forward)
// ---------------------------------------------------------------------------
template <int DT>
__global__ void __launch_bounds__(256) sparse_query_kernel(const nglod_sparse_model m, const uint8_t *__restrict__ oct,
                                                           const uint32_t *__restrict__ prefix, int lod,
                                                           const float *__restrict__ x, int64_t n,
                                                           float *__restrict__ out) {
    extern __shared__ float4 smem[];
    const int H = m.hidden_dim;
    stage_decoder_ptrs(smem, H, m.w0[lod], m.b0[lod], m.w1[lod], m.b1[lod]);
    __syncthreads();
    const int level = lod + 2;
    const float res = (float)(1 << level);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
        const float ux = fmaf(px, 0.5f, 0.5f) * res, uy = fmaf(py, 0.5f, 0.5f) * res,
                    uz = fmaf(pz, 0.5f, 0.5f) * res;
        bool found = ux >= 0.f && uy >= 0.f && uz >= 0.f && ux < res && uy < res && uz < res;
        int64_t ord = 0;
        if (found) {
            const uint32_t vx = (uint32_t)ux, vy = (uint32_t)uy, vz = (uint32_t)uz;
            for (int l = 0; l < level && found; ++l) {
                const int depth = level - l - 1;
                const uint32_t child = (((vx >> depth) & 1u) << 2) | (((vy >> depth) & 1u) << 1) | ((vz >> depth) & 1u);
                const uint32_t bits = oct[ord];
                if (!(bits & (1u << child))) {
                    found = false;
                } else {
                    ord = (int64_t)prefix[ord] + __popc(bits & ((2u << child) - 1u));
                }
            }
        }
        float f[kC];
        sparse_features<DT>(m, lod, found ? ord : m.level_start[level], px, py, pz, f);
        const float d = decode_f32(smem, H, px, py, pz, f);
        out[i] = found ? d : __int_as_float(0x7fc00000);
    }
}

// ---------------------------------------------------------------------------
// construction
// ---------------------------------------------------------------------------
// Dense corner grid of one level: flag[(x*s + y)*s + z] = 1 for every corner
// of an occupied voxel.
__global__ void mark_corners_kernel(const short4 *__restrict__ pts, int64_t start, int64_t cnt, int s,
                                    uint8_t *__restrict__ flag) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride) {
        const short4 p = pts[start + k];
        for (int j = 0; j < 8; ++j) {
            const int cx = p.x + ((j >> 2) & 1), cy = p.y + ((j >> 1) & 1), cz = p.z + (j & 1);
            flag[((int64_t)cx * s + cy) * s + cz] = 1;
        }
    }
}

__global__ void __launch_bounds__(kChunk) flag_chunk_kernel(const uint8_t *__restrict__ flag, const int64_t *count,
                                                            uint32_t *partials) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t s = block_sum((i < n && flag[i]) ? 1u : 0u, s_warp);
        if (threadIdx.x == 0) partials[c] = s;
    }
}

// ids[i] = global corner index of grid cell i (or -1); features copied from
// the channel-last dense volume (index ((z*s + y)*s + x)*C).
template <int DT>
__global__ void __launch_bounds__(kChunk) corner_emit_kernel(const uint8_t *__restrict__ flag, const int64_t *count,
                                                             const uint32_t *partials, int s, int64_t offset,
                                                             int32_t *__restrict__ ids, const float *__restrict__ vol,
                                                             void *feats, int64_t cap, int64_t *status) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && flag[i]) ? 1u : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(f, s_warp, &tot);
        if (i >= n) continue;
        if (!f) {
            ids[i] = -1;
            continue;
        }
        const int64_t k = offset + (int64_t)partials[c] + ex;
        if (k >= cap) {
            *status = 1;
            ids[i] = -1;
            continue;
        }
        ids[i] = (int32_t)k;
        const int64_t cz = i % s, cy = (i / s) % s, cx = i / ((int64_t)s * s);
        const float *src = vol + ((cz * s + cy) * s + cx) * kC;
        if (DT == NGLOD_F32) {
            float *dst = static_cast<float *>(feats) + k * kC;
            for (int q = 0; q < kC; ++q) dst[q] = src[q];
        } else {
            __nv_bfloat16 *dst = static_cast<__nv_bfloat16 *>(feats) + k * kC;
            for (int q = 0; q < kC; ++q) dst[q] = __float2bfloat16_rn(src[q]);
        }
    }
}

__global__ void trinket_kernel(const short4 *__restrict__ pts, int64_t start, int64_t cnt, int s,
                               const int32_t *__restrict__ ids, const int32_t *__restrict__ pgrid, int ps,
                               int32_t *__restrict__ corner_idx, int32_t *__restrict__ parent) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride) {
        const int64_t g = start + k;
        const short4 p = pts[g];
        for (int j = 0; j < 8; ++j) {
            const int cx = p.x + ((j >> 2) & 1), cy = p.y + ((j >> 1) & 1), cz = p.z + (j & 1);
            corner_idx[8 * g + j] = ids[((int64_t)cx * s + cy) * s + cz];
        }
        parent[g] = pgrid ? pgrid[((int64_t)(p.x >> 1) * ps + (p.y >> 1)) * ps + (p.z >> 1)] : -1;
    }
}

__global__ void point_grid_kernel(const short4 *__restrict__ pts, int64_t start, int64_t cnt, int s,
                                  int32_t *__restrict__ grid) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride) {
        const short4 p = pts[start + k];
        grid[((int64_t)p.x * s + p.y) * s + p.z] = (int32_t)(start + k);
    }
}

inline int sgrid(int64_t n, int threads = 256) {
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)num_sms() * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

inline int64_t cube(int64_t s) { return s * s * s; }

inline int check_sparse_model(const nglod_sparse_model *m, int lod) {
    NGLOD_REQUIRE(m != nullptr, NGLOD_ERR_INVALID, "sparse model is null");
    NGLOD_REQUIRE(m->num_lods >= 1 && m->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID, "num_lods=%d", m->num_lods);
    NGLOD_REQUIRE(lod >= 0 && lod < m->num_lods && lod + 2 < 16, NGLOD_ERR_INVALID, "lod=%d outside [0, %d)", lod,
                  m->num_lods);
    NGLOD_REQUIRE(m->feature_dim == kC, NGLOD_ERR_UNSUPPORTED, "feature_dim=%d not built", m->feature_dim);
    NGLOD_REQUIRE(m->hidden_dim >= 2 && m->hidden_dim <= 256 && m->hidden_dim % 2 == 0, NGLOD_ERR_UNSUPPORTED,
                  "hidden_dim=%d not built", m->hidden_dim);
    NGLOD_REQUIRE(m->feat_dtype == NGLOD_F32 || m->feat_dtype == NGLOD_BF16, NGLOD_ERR_UNSUPPORTED,
                  "feat_dtype=%d", m->feat_dtype);
    NGLOD_REQUIRE(m->corner_feats && m->corner_idx && m->parent && m->points && m->w0[lod] && m->b0[lod] &&
                      m->w1[lod] && m->b1[lod],
                  NGLOD_ERR_INVALID, "sparse model has a null pointer");
    NGLOD_REQUIRE(aligned(m->corner_feats, 16) && aligned(m->corner_idx, 16) && aligned(m->points, 8),
                  NGLOD_ERR_ALIGN, "corner_feats/corner_idx must be 16-byte and points 8-byte aligned");
    return NGLOD_OK;
}

}  // namespace nglod

using namespace nglod;

extern "C" int64_t nglod_sparse_build_scratch_bytes(int32_t level) {
    if (level < 2 || level > 9) return -1;
    const int64_t s = ((int64_t)1 << level) + 1;
    const int64_t ps = (int64_t)1 << (level - 1);
    const int64_t flags = (cube(s) + 255) & ~(int64_t)255;
    const int64_t ids = (cube(s) * 4 + 255) & ~(int64_t)255;
    const int64_t pg = (cube(ps) * 4 + 255) & ~(int64_t)255;
    const int64_t parts = ((cube(s) / kChunk + 2) * 4 + 255) & ~(int64_t)255;
    return flags + ids + pg + parts + 8 * 8;
}

extern "C" int nglod_sparse_build(const nglod_dense_model *dense, const int16_t *points, const int32_t *pyramid_host,
                                  int32_t level, int32_t feat_dtype, void *corner_feats, int64_t corner_cap,
                                  int32_t *corner_idx, int32_t *parent, int64_t *corner_counts_host, void *scratch,
                                  nglod_stream_t stream) {
    NGLOD_REQUIRE(dense != nullptr, NGLOD_ERR_INVALID, "dense model is null");
    NGLOD_TRY(check_model(dense, dense->num_lods - 1));
    NGLOD_REQUIRE(dense->base_lod == 2, NGLOD_ERR_UNSUPPORTED,
                  "sparse export needs base_lod=2 (LOD i on octree level i+2), got %d", dense->base_lod);
    const int nl = dense->num_lods;
    NGLOD_REQUIRE(level >= nl + 1 && nl + 1 <= 9, NGLOD_ERR_INVALID,
                  "octree level=%d must be >= num_lods+1=%d (and num_lods+1 <= 9)", level, nl + 1);
    NGLOD_REQUIRE(feat_dtype == NGLOD_F32 || feat_dtype == NGLOD_BF16, NGLOD_ERR_UNSUPPORTED, "feat_dtype=%d",
                  feat_dtype);
    NGLOD_REQUIRE(points && pyramid_host && corner_feats && corner_idx && parent && corner_counts_host && scratch,
                  NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(scratch, 256) && aligned(points, 8), NGLOD_ERR_ALIGN, "scratch/points alignment");
    cudaStream_t st = (cudaStream_t)stream;
    const int32_t *psum = pyramid_host + (level + 2);
    const short4 *pts = reinterpret_cast<const short4 *>(points);
    const int maxlv = nl + 1;
    const int64_t smax = ((int64_t)1 << maxlv) + 1;
    uint8_t *base = static_cast<uint8_t *>(scratch);
    uint8_t *flag = base;
    int32_t *ids = reinterpret_cast<int32_t *>(base + ((cube(smax) + 255) & ~(int64_t)255));
    int32_t *pgrid = reinterpret_cast<int32_t *>(reinterpret_cast<uint8_t *>(ids) +
                                                 ((cube(smax) * 4 + 255) & ~(int64_t)255));
    const int64_t psmax = (int64_t)1 << (maxlv - 1);
    uint32_t *partials =
        reinterpret_cast<uint32_t *>(reinterpret_cast<uint8_t *>(pgrid) + ((cube(psmax) * 4 + 255) & ~(int64_t)255));
    int64_t *ctrl = reinterpret_cast<int64_t *>(reinterpret_cast<uint8_t *>(partials) +
                                                (((cube(smax) / kChunk + 2) * 4 + 255) & ~(int64_t)255));
    NGLOD_TRY(cuda_status(cudaMemsetAsync(ctrl, 0, 8 * sizeof(int64_t), st), "sparse build memset"));
    int64_t offset = 0;
    for (int i = 0; i < nl; ++i) {
        const int lv = i + 2;
        const int s = (1 << lv) + 1;
        const int64_t start = psum[lv], cnt = psum[lv + 1] - psum[lv];
        const int64_t ncell = cube(s);
        NGLOD_TRY(cuda_status(cudaMemsetAsync(flag, 0, (size_t)ncell, st), "sparse build memset"));
        mark_corners_kernel<<<sgrid(cnt), 256, 0, st>>>(pts, start, cnt, s, flag);
        NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl + 2, &ncell, sizeof(int64_t), cudaMemcpyHostToDevice, st),
                              "sparse build copy"));
        const int64_t chunks = (ncell + kChunk - 1) / kChunk;
        const int grid = (int)(chunks < num_sms() * 2 ? chunks : num_sms() * 2);
        flag_chunk_kernel<<<grid, kChunk, 0, st>>>(flag, ctrl + 2, partials);
        scan_chunk_counts_kernel<<<1, kChunk, 0, st>>>(partials, ctrl + 2, ctrl + 3, INT64_MAX, nullptr);
        if (feat_dtype == NGLOD_F32)
            corner_emit_kernel<NGLOD_F32><<<grid, kChunk, 0, st>>>(flag, ctrl + 2, partials, s, offset, ids,
                                                                   static_cast<const float *>(dense->grid[i]),
                                                                   corner_feats, corner_cap, ctrl);
        else
            corner_emit_kernel<NGLOD_BF16><<<grid, kChunk, 0, st>>>(flag, ctrl + 2, partials, s, offset, ids,
                                                                    static_cast<const float *>(dense->grid[i]),
                                                                    corner_feats, corner_cap, ctrl);
        const int ps = 1 << (lv - 1);
        if (lv > 2) {
            NGLOD_TRY(cuda_status(cudaMemsetAsync(pgrid, 0xff, (size_t)cube(ps) * 4, st), "sparse build memset"));
            point_grid_kernel<<<sgrid(psum[lv] - psum[lv - 1]), 256, 0, st>>>(pts, psum[lv - 1],
                                                                              psum[lv] - psum[lv - 1], ps, pgrid);
        }
        trinket_kernel<<<sgrid(cnt), 256, 0, st>>>(pts, start, cnt, s, ids, lv > 2 ? pgrid : nullptr, ps, corner_idx,
                                                   parent);
        NGLOD_TRY(launch_status("nglod_sparse_build"));
        int64_t c = 0;
        NGLOD_TRY(cuda_status(cudaMemcpyAsync(&c, ctrl + 3, sizeof(int64_t), cudaMemcpyDeviceToHost, st),
                              "sparse build copy"));
        NGLOD_TRY(cuda_status(cudaStreamSynchronize(st), "sparse build sync"));
        corner_counts_host[i] = c;
        offset += c;
    }
    int64_t status = 0;
    NGLOD_TRY(cuda_status(cudaMemcpy(&status, ctrl, sizeof(int64_t), cudaMemcpyDeviceToHost), "sparse build copy"));
    NGLOD_REQUIRE(status == 0 && offset <= corner_cap, NGLOD_ERR_CAPACITY,
                  "sparse build needs %lld corner rows, capacity %lld", (long long)offset, (long long)corner_cap);
    return NGLOD_OK;
}

extern "C" int nglod_sparse_query(const nglod_sparse_model *model, const uint8_t *octree, const uint32_t *prefix,
                                  int32_t lod, const float *x, int64_t n, float *out, nglod_stream_t stream) {
    NGLOD_TRY(check_sparse_model(model, lod));
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(octree && prefix && x && out, NGLOD_ERR_INVALID, "null pointer argument");
    const size_t smem = (size_t)decoder_f4(model->hidden_dim) * sizeof(float4);
    const int threads = 256;
    const int64_t want = (n + threads - 1) / threads;
    if (model->feat_dtype == NGLOD_F32) {
        auto k = sparse_query_kernel<NGLOD_F32>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, (cudaStream_t)stream>>>(*model, octree, prefix, lod, x, n,
                                                                                   out);
    } else {
        auto k = sparse_query_kernel<NGLOD_BF16>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, (cudaStream_t)stream>>>(*model, octree, prefix, lod, x, n,
                                                                                   out);
    }
    return launch_status("nglod_sparse_query");
}

extern "C" int nglod_sparse_trace_tc(const nglod_sparse_model *model, int32_t lod, int32_t num_steps,
                                     const float *ray_o, const float *ray_d, int64_t n, const int32_t *nuggets,
                                     int64_t n_nuggets, int32_t *ray_first, float *x, float *t, uint8_t *hit,
                                     float *normal, int64_t *work_counter, int32_t *status, nglod_stream_t stream) {
    NGLOD_TRY(check_sparse_model(model, lod));
    NGLOD_REQUIRE(model->feat_dtype == NGLOD_BF16 && model->feature_dim == kC && model->hidden_dim == kHid,
                  NGLOD_ERR_UNSUPPORTED, "tensor-core sparse trace built for bf16 corner features, C=32, H=128");
    NGLOD_REQUIRE(model->w0_tile[lod] && aligned(model->w0_tile[lod], 16) && aligned(model->corner_feats, 16),
                  NGLOD_ERR_ALIGN, "decoder tile %d / corner features null or not 16-byte aligned", lod);
    NGLOD_REQUIRE(n >= 0 && n_nuggets >= 0 && num_steps >= 0, NGLOD_ERR_INVALID, "negative size");
    // global voxel indices travel as int32 through shared memory: the level's
    // first index plus its at most 8^level voxels must stay below 2^31
    NGLOD_REQUIRE(lod + 2 <= 9 && model->level_start[lod + 2] + ((int64_t)1 << (3 * (lod + 2))) < ((int64_t)1 << 31),
                  NGLOD_ERR_UNSUPPORTED, "voxel indices of level %d must fit 31 bits", lod + 2);
    NGLOD_REQUIRE(!model->corner_chain[lod] || aligned(model->corner_chain[lod], 16), NGLOD_ERR_ALIGN,
                  "corner_chain %d is not 16-byte aligned", lod);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && ray_first && x && t && hit && work_counter && status && (nuggets || n_nuggets == 0),
                  NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(work_counter, 8) && (n_nuggets == 0 || aligned(nuggets, 8)), NGLOD_ERR_ALIGN,
                  "work_counter and nuggets must be 8-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int32_t), st), "sparse trace memset"));
    NGLOD_TRY(cuda_status(cudaMemsetAsync(ray_first, 0xff, (size_t)n * sizeof(int32_t), st), "sparse trace memset"));
    if (n_nuggets > 0)
        ray_first_kernel<<<sgrid(n_nuggets), 256, 0, st>>>(reinterpret_cast<const int2 *>(nuggets), n_nuggets,
                                                           ray_first);
    NGLOD_TRY(cuda_status(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), st), "sparse trace memset"));
    SparseTcArgs a;
    a.t.m = *model;
    a.t.lod = lod;
    a.t.num_steps = num_steps;
    a.t.ray_o = ray_o;
    a.t.ray_d = ray_d;
    a.t.n = n;
    a.t.nug = reinterpret_cast<const int2 *>(nuggets);
    a.t.n_nug = n_nuggets;
    a.t.ray_first = ray_first;
    a.t.x = x;
    a.t.t = t;
    a.t.hit = hit;
    a.t.normal = normal;
    a.t.counter = reinterpret_cast<unsigned long long *>(work_counter);
    a.status = status;
    auto kernel = model->corner_chain[lod] ? sparse_trace_tc_kernel<true> : sparse_trace_tc_kernel<false>;
    NGLOD_TRY(cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes),
                          "cudaFuncSetAttribute"));
    const int64_t want = (n + kTP - 1) / kTP;
    const int64_t cap = (int64_t)num_sms() * 4;
    kernel<<<(int)(want < cap ? want : cap), kTP, kSmemBytes, st>>>(a);
    return launch_status("nglod_sparse_trace_tc");
}

extern "C" int nglod_sparse_build_chain(const nglod_sparse_model *model, int32_t lod, int64_t count, int32_t *chain,
                                        nglod_stream_t stream) {
    NGLOD_REQUIRE(model != nullptr, NGLOD_ERR_INVALID, "model is null");
    NGLOD_REQUIRE(lod >= 0 && lod < model->num_lods && lod + 3 < 16, NGLOD_ERR_INVALID, "lod=%d", lod);
    NGLOD_REQUIRE(count == model->level_start[lod + 3] - model->level_start[lod + 2], NGLOD_ERR_INVALID,
                  "count=%lld is not the number of level-%d voxels (%lld)", (long long)count, lod + 2,
                  (long long)(model->level_start[lod + 3] - model->level_start[lod + 2]));
    if (count == 0) return NGLOD_OK;
    NGLOD_REQUIRE(model->corner_idx && model->parent && chain, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(model->corner_idx, 16) && aligned(chain, 16), NGLOD_ERR_ALIGN,
                  "corner_idx and chain must be 16-byte aligned");
    chain_build_kernel<<<sgrid(count), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const int4 *>(model->corner_idx), model->parent, model->level_start[lod + 2], count, lod,
        reinterpret_cast<int4 *>(chain));
    return launch_status("nglod_sparse_build_chain");
}

extern "C" int nglod_sparse_trace(const nglod_sparse_model *model, int32_t lod, int32_t num_steps, const float *ray_o,
                                  const float *ray_d, int64_t n, const int32_t *nuggets, int64_t n_nuggets,
                                  int32_t *ray_first, float *x, float *t, uint8_t *hit, float *normal,
                                  int64_t *work_counter, nglod_stream_t stream) {
    NGLOD_TRY(check_sparse_model(model, lod));
    NGLOD_REQUIRE(n >= 0 && n_nuggets >= 0 && num_steps >= 0, NGLOD_ERR_INVALID, "negative size");
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && ray_first && x && t && hit && work_counter && (nuggets || n_nuggets == 0),
                  NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(work_counter, 8) && (n_nuggets == 0 || aligned(nuggets, 8)), NGLOD_ERR_ALIGN,
                  "work_counter and nuggets must be 8-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemsetAsync(ray_first, 0xff, (size_t)n * sizeof(int32_t), st), "sparse trace memset"));
    if (n_nuggets > 0)
        ray_first_kernel<<<sgrid(n_nuggets), 256, 0, st>>>(reinterpret_cast<const int2 *>(nuggets), n_nuggets,
                                                           ray_first);
    NGLOD_TRY(cuda_status(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), st), "sparse trace memset"));
    SparseTraceArgs a;
    a.m = *model;
    a.lod = lod;
    a.num_steps = num_steps;
    a.ray_o = ray_o;
    a.ray_d = ray_d;
    a.n = n;
    a.nug = reinterpret_cast<const int2 *>(nuggets);
    a.n_nug = n_nuggets;
    a.ray_first = ray_first;
    a.x = x;
    a.t = t;
    a.hit = hit;
    a.normal = normal;
    a.counter = reinterpret_cast<unsigned long long *>(work_counter);
    const int threads = 128;
    const size_t smem = (size_t)decoder_f4(model->hidden_dim) * sizeof(float4);
    const int64_t want = (n + threads - 1) / threads;
    if (model->feat_dtype == NGLOD_F32) {
        auto k = sparse_trace_kernel<NGLOD_F32>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, st>>>(a);
    } else {
        auto k = sparse_trace_kernel<NGLOD_BF16>;
        NGLOD_TRY(prepare_smem(k, smem));
        const int64_t cap = resident_blocks(k, threads, smem);
        k<<<(int)(want < cap ? want : cap), threads, smem, st>>>(a);
    }
    return launch_status("nglod_sparse_trace");
}
