// Structured point cloud (SPC) octree: build from voxels, decode, and the
// level-by-level ray/octree traversal of sol-renderer's spc_raytrace.
//
// Every variable-length step is a stream compaction done with "chunk scans":
// a chunk is 1024 consecutive elements handled by one 1024-thread block
// iteration; pass 1 reduces each chunk to a count, pass 2 (one block) turns
// the counts into exclusive chunk offsets and the total, pass 3 rescans each
// chunk and writes its survivors.  Element counts of every level live in a
// small device control block, so the traversal of all levels is enqueued
// without any host round trip; the host reads the result once at the end.
#include <stdio.h>

#include <vector>

#include "scan.cuh"

namespace nglod {

constexpr int kMaxSpcLevels = 15;
constexpr int kCtrlStatus = 0;   // 0 ok, 1 capacity exceeded
constexpr int kCtrlCount = 4;    // count of level l at kCtrlCount + l

// ---------------------------------------------------------------------------
// front-to-back child order
// ---------------------------------------------------------------------------
// Children of a voxel visited by a ray whose origin lies in octant `code`
// (4*[x > centre] + 2*[y > centre] + [z > centre]) come nearest first: sorted
// by the Hamming distance of their octant index to `code`, ties by index.
// This reproduces the Order table of spc_raytrace_cuda_kernel.cu:39-47.
// The order of a code packed 3 bits per rank (rank 0 in the low bits).
constexpr uint32_t popc3(uint32_t v) { return (v & 1u) + ((v >> 1) & 1u) + ((v >> 2) & 1u); }
constexpr uint32_t order_word(uint32_t code) {
    uint32_t w = 0, r = 0;
    for (uint32_t dist = 0; dist <= 3; ++dist)
        for (uint32_t j = 0; j < 8; ++j)
            if (popc3(j ^ code) == dist) w |= j << (3 * r++);
    return w;
}
static_assert(order_word(0) == (0u | 1u << 3 | 2u << 6 | 4u << 9 | 3u << 12 | 5u << 15 | 6u << 18 | 7u << 21),
              "child order of octant 0");
__constant__ uint32_t c_child_order[8] = {order_word(0), order_word(1), order_word(2), order_word(3),
                                          order_word(4), order_word(5), order_word(6), order_word(7)};

// ---------------------------------------------------------------------------
// ray / voxel test (d_Decide, d_FaceEval of spc_raytrace_cuda_kernel.cu:85-138)
// ---------------------------------------------------------------------------
// The ray is mapped to [0,1]^3 (o' = o/2 + 1/2, d' = d/2); the voxel (i, j)
// square of each coordinate plane is tested against the line's 2-D edge
// function a*i + b*j + c at its four corners.  Arithmetic order: the
// reference source as nvcc contracts it, i.e. c0 = fma(b, j, a*i) + c,
// c1 = c0 + a, c2 = c0 + b, c3 = c1 + b, and o' x d' with each component
// fma(u, v, -(w*z)).  This form was pinned against the reference kernel
// itself: of the nine legal contractions of the two expressions, only this
// one reproduces all of its decisions on 135M ray/voxel candidates (a
// 1920x1080 frame through a level-7 octree).
// The reference keeps a running min (from 1) and max (from -1) of the four
// corner values, skipping NaNs, and tests min <= 0 and max >= 0; that is
// "some value <= 0 and some value >= 0", which fminf / fmaxf (a NaN operand
// yields the other one; all NaN gives NaN, which fails both tests) decide in
// six min / max operations.
__device__ __forceinline__ bool face_straddles(float fi, float fj, float a, float b, float c) {
    const float r0 = __fadd_rn(__fmaf_rn(b, fj, __fmul_rn(a, fi)), c);
    const float r1 = __fadd_rn(r0, a);
    const float r2 = __fadd_rn(r0, b);
    const float r3 = __fadd_rn(r1, b);
    const float mn = fminf(fminf(r0, r1), fminf(r2, r3));
    const float mx = fmaxf(fmaxf(r0, r1), fmaxf(r2, r3));
    return mn <= 0.f && mx >= 0.f;
}

// 2^e as a float for -126 <= e <= 127 (exact: the exponent field alone).
// Multiplying by it equals ldexpf for normal results, as all of them are
// here (levels <= 15, coordinates >= 0.5 * 2^-15).
__device__ __forceinline__ float pow2i(int e) { return __int_as_float((127 + e) << 23); }

// The three edge functions (a, b, c per plane) of one ray at one level.
struct RayFaces {
    float a0, b0, c0, a1, b1, c1, a2, b2, c2;
};

__device__ __forceinline__ RayFaces ray_faces(const float *__restrict__ org, const float *__restrict__ dir,
                                              uint32_t ridx, int level) {
    const float ox = __fmaf_rn(0.5f, org[3 * ridx], 0.5f);
    const float oy = __fmaf_rn(0.5f, org[3 * ridx + 1], 0.5f);
    const float oz = __fmaf_rn(0.5f, org[3 * ridx + 2], 0.5f);
    const float dx = __fmul_rn(0.5f, dir[3 * ridx]);
    const float dy = __fmul_rn(0.5f, dir[3 * ridx + 1]);
    const float dz = __fmul_rn(0.5f, dir[3 * ridx + 2]);
    const float cx = __fmaf_rn(oy, dz, -__fmul_rn(dy, oz));
    const float cy = __fmaf_rn(oz, dx, -__fmul_rn(dz, ox));
    const float cz = __fmaf_rn(ox, dy, -__fmul_rn(dx, oy));
    const float s1 = pow2i(-level);
    const float s2 = __fmul_rn(s1, s1);
    RayFaces f;
    f.a0 = __fmul_rn(-s2, dz);
    f.b0 = __fmul_rn(s2, dy);
    f.c0 = __fmul_rn(s1, cx);
    f.a1 = __fmul_rn(s2, dz);
    f.b1 = __fmul_rn(-s2, dx);
    f.c1 = __fmul_rn(s1, cy);
    f.a2 = __fmul_rn(-s2, dy);
    f.b2 = __fmul_rn(s2, dx);
    f.c2 = __fmul_rn(s1, cz);
    return f;
}

// Voxel (px, py, pz) (integer coordinates at the faces' level, exact in float).
__device__ __forceinline__ bool faces_hit(const RayFaces &f, float px, float py, float pz) {
    return face_straddles(py, pz, f.a0, f.b0, f.c0) && face_straddles(px, pz, f.a1, f.b1, f.c1) &&
           face_straddles(px, py, f.a2, f.b2, f.c2);
}

__device__ __forceinline__ bool ray_hits_voxel(const float *__restrict__ org, const float *__restrict__ dir,
                                               uint32_t ridx, short4 p, int level) {
    return faces_hit(ray_faces(org, dir, ridx, level), (float)(unsigned short)p.x, (float)(unsigned short)p.y,
                     (float)(unsigned short)p.z);
}

// Octant of the ray origin relative to the voxel centre (d_Subdivide,
// spc_raytrace_cuda_kernel.cu:157-167).  The reference forms
// a - v = (0.5*o + 0.5) - scale*(p + 0.5) in double and tests the float of it
// for > 0.  a is a float and v = 2^-level * (p + 0.5) is exact in float
// (p < 2^15), both are multiples of 2^-149, so a - v is zero or at least
// 2^-149 in magnitude: its float keeps its sign, and the test is a > v,
// evaluated here in float (NaN origins compare false either way).
__device__ __forceinline__ uint32_t origin_octant(const float *__restrict__ org, uint32_t ridx, short4 p,
                                                  int level) {
    const float ax = __fmaf_rn(0.5f, org[3 * ridx], 0.5f);
    const float ay = __fmaf_rn(0.5f, org[3 * ridx + 1], 0.5f);
    const float az = __fmaf_rn(0.5f, org[3 * ridx + 2], 0.5f);
    const float sc = pow2i(-level);
    const float vx = __fmul_rn((float)p.x + 0.5f, sc);
    const float vy = __fmul_rn((float)p.y + 0.5f, sc);
    const float vz = __fmul_rn((float)p.z + 0.5f, sc);
    return (ax > vx ? 4u : 0u) + (ay > vy ? 2u : 0u) + (az > vz ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// traversal kernel
// ---------------------------------------------------------------------------
// Level l's pass turns the nuggets of level l (voxels the ray is known to
// hit; at level 0 every ray with the root, tested here) into the nuggets of
// level l+1: the children of each voxel that are occupied and hit by the
// ray, nearest first.  One launch per level, one 1024-nugget chunk per block
// iteration: the block tests its nuggets' children (hit mask and origin
// octant per nugget, kept in registers), scans the hit counts, finds the
// chunk's output offset by a decoupled look-back over the preceding chunks'
// published counts, and writes the hit children in the octant's order.
// This produces the reference's nuggets exactly: the reference emits every
// occupied child and drops the missed ones at the next level, which leaves
// the same children in the same order.
//
// Chunks are taken in ticket order (one atomic per block iteration), so a
// chunk's predecessors belong to blocks that are already running and
// publish their counts without waiting on anything; the look-back reads 32
// predecessors' states per step, each wait is bounded (kLookbackPolls), and
// a wait that gives up raises the status (kStatusLookback) instead of
// hanging.
struct TraverseArgs {
    const uint8_t *octree;
    const short4 *points;  // all levels
    const uint32_t *prefix;
    const float *org;
    const float *dir;
    const int2 *in;  // nuggets of this level (unused at level 0)
    int2 *out;
    unsigned long long *state;  // this level's chunk states
    uint32_t *ticket;           // this level's chunk ticket
    int64_t *ctrl;
    int64_t capacity;
    int level;       // current level
    int target;      // target level (== level only for the root-only pass of target 0)
    int64_t off0;    // global point index of this level's first point
    int64_t off1;    // ... of the next level's
};

// Chunk state word: flag in bits 32-33 (kStateCount: the chunk's own hit
// count; kStatePrefix: its inclusive prefix), the value in bits 0-31.
constexpr unsigned long long kStateCount = 1ull << 32, kStatePrefix = 2ull << 32;
constexpr uint32_t kLookbackPolls = 1u << 22;
constexpr int64_t kStatusLookback = 2;
// Scratch of nglod_spc_raytrace in its `info` buffer: 16 tickets, then the
// chunk states of each pass.
constexpr int64_t kTicketBytes = 64;
inline int64_t state_words(int64_t capacity) { return (capacity + kChunk - 1) / kChunk + 1; }

__device__ __forceinline__ int2 nugget_at(const TraverseArgs &a, int64_t i) {
    if (a.level == 0) return make_int2((int)i, 0);
    return a.in[i];
}

// One nugget's decision: the hit mask (bits 0-7, by child index) and the
// origin octant (bits 8-10); its octree byte and point index for the emit.
__device__ __forceinline__ uint32_t decide_nugget(const TraverseArgs &a, int2 nug, uint32_t &o, int64_t &node) {
    node = a.off0 + nug.y;
    const short4 p = a.points[node];
    uint32_t inf = 0;
    if (a.level > 0 || ray_hits_voxel(a.org, a.dir, (uint32_t)nug.x, p, 0)) {
        if (a.level == a.target) {
            inf = 1u;
        } else {
            o = a.octree[node];
            const RayFaces f = ray_faces(a.org, a.dir, (uint32_t)nug.x, a.level + 1);
            const float bx = (float)(2 * (int)p.x), by = (float)(2 * (int)p.y), bz = (float)(2 * (int)p.z);
            // A child's three plane tests depend on two of its three
            // coordinates each, so the eight children need twelve distinct
            // tests (the same expressions on the same inputs as testing
            // every child alone); all twelve run, without branches.
            uint32_t m0 = 0, m1 = 0, m2 = 0;
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    m0 |= (uint32_t)face_straddles(by + (float)u, bz + (float)w, f.a0, f.b0, f.c0) << (2 * u + w);
                    m1 |= (uint32_t)face_straddles(bx + (float)u, bz + (float)w, f.a1, f.b1, f.c1) << (2 * u + w);
                    m2 |= (uint32_t)face_straddles(bx + (float)u, by + (float)w, f.a2, f.b2, f.c2) << (2 * u + w);
                }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int dx = (j >> 2) & 1, dy = (j >> 1) & 1, dz = j & 1;
                inf |= ((o >> j) & (m0 >> (2 * dy + dz)) & (m1 >> (2 * dx + dz)) & (m2 >> (2 * dx + dy)) & 1u) << j;
            }
            inf |= origin_octant(a.org, (uint32_t)nug.x, p, a.level) << 8;
        }
    }
    return inf;
}

// 256 threads per block, four consecutive nuggets of a 1024-nugget chunk
// per thread (decided one after the other, so a warp's divergence averages
// over four decisions, and a chunk costs a 256-thread scan).
constexpr int kTravThreads = 256, kTravPer = kChunk / kTravThreads;

__global__ void __launch_bounds__(kTravThreads, 4) traverse_level_kernel(const TraverseArgs a) {
    __shared__ uint32_t s_warp[kTravThreads / 32 + 1];
    __shared__ uint32_t s_order[8];
    __shared__ int64_t s_chunk;
    __shared__ uint32_t s_excl;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 8) s_order[tid] = c_child_order[tid];
    const int64_t count = a.ctrl[kCtrlCount + a.level];
    const int64_t nchunks = (count + kChunk - 1) / kChunk;
    // an empty level has no last chunk to write the next level's count
    if (nchunks == 0 && blockIdx.x == 0 && tid == 0) a.ctrl[kCtrlCount + a.level + 1] = 0;
    volatile unsigned long long *st = a.state;
    for (;;) {
        if (tid == 0) {
            const int64_t c = (int64_t)atomicAdd(a.ticket, 1u);
            // after a raised status (an earlier level overflowed, or a wait
            // gave up) nothing more is read or written
            s_chunk = *(volatile int64_t *)(a.ctrl + kCtrlStatus) != 0 ? nchunks : c;
        }
        __syncthreads();
        const int64_t c = s_chunk;
        if (c >= nchunks) break;
        // 1. decide this thread's four nuggets
        const int64_t i0 = c * kChunk + (int64_t)tid * kTravPer;
        uint32_t inf[kTravPer], oct[kTravPer];
        int2 nug[kTravPer];
        int64_t node[kTravPer];
        uint32_t v = 0;
#pragma unroll
        for (int e = 0; e < kTravPer; ++e) {
            inf[e] = 0;
            oct[e] = 0;
            node[e] = 0;
            nug[e] = make_int2(0, 0);
            if (i0 + e < count) {
                nug[e] = nugget_at(a, i0 + e);
                inf[e] = decide_nugget(a, nug[e], oct[e], node[e]);
            }
            v += (uint32_t)__popc(inf[e] & 0xffu);
        }
        // 2. exclusive scan of the threads' hit counts
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = lane < kTravThreads / 32 ? s_warp[lane] : 0u;
            uint32_t wi = w;
#pragma unroll
            for (int o = 1; o < kTravThreads / 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            if (lane < kTravThreads / 32) s_warp[lane] = wi - w;  // exclusive prefix of warp totals
            if (lane == kTravThreads / 32 - 1) s_warp[kTravThreads / 32] = wi;
        }
        __syncthreads();
        const uint32_t ex = s_warp[warp] + x - v;
        const uint32_t tot = s_warp[kTravThreads / 32];
        // 3. the chunk's offset: publish its count, then warp 0 adds the
        // predecessors' counts 32 chunks at a time, back to the nearest chunk
        // that has published its inclusive prefix
        if (warp == 0) {
            uint32_t excl = 0;
            if (c == 0) {
                if (lane == 0) st[0] = kStatePrefix | tot;
            } else {
                if (lane == 0) st[c] = kStateCount | tot;
                int64_t k = c - 1;
                uint32_t polls = 0;
                bool failed = false;
                for (;;) {
                    const int64_t idx = k - lane;
                    unsigned long long w = kStatePrefix;  // before chunk 0: an empty prefix
                    if (idx >= 0) w = st[idx];
                    const unsigned pmask = __ballot_sync(0xffffffffu, (w & kStatePrefix) != 0);
                    const unsigned dmask = __ballot_sync(0xffffffffu, (w & (kStatePrefix | kStateCount)) != 0);
                    const int jp = pmask ? __ffs(pmask) - 1 : 32;  // nearest inclusive prefix
                    const unsigned need = jp == 32 ? 0xffffffffu : (2u << jp) - 1u;
                    if ((dmask & need) == need) {
                        uint32_t val = lane <= jp ? (uint32_t)w : 0u;
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
                        excl += val;
                        if (jp < 32) break;
                        k -= 32;
                        polls = 0;
                    } else if (++polls > kLookbackPolls) {
                        failed = true;
                        break;
                    } else if (polls > 32) {
                        __nanosleep(64);
                    }
                }
                if (lane == 0) {
                    if (failed)
                        atomicExch(reinterpret_cast<unsigned long long *>(a.ctrl + kCtrlStatus),
                                   (unsigned long long)kStatusLookback);
                    st[c] = kStatePrefix | (excl + tot);
                }
            }
            if (lane == 0) {
                s_excl = excl;
                if (c == nchunks - 1) {
                    const int64_t total = (int64_t)excl + tot;
                    a.ctrl[kCtrlCount + a.level + 1] = total;
                    if (total > a.capacity)
                        atomicExch(reinterpret_cast<unsigned long long *>(a.ctrl + kCtrlStatus), 1ull);
                }
            }
        }
        __syncthreads();
        // 4. emit the hit children nearest first (nothing beyond the capacity)
        int64_t pos = (int64_t)s_excl + ex;
        if (v != 0 && pos + v <= a.capacity) {
#pragma unroll
            for (int e = 0; e < kTravPer; ++e) {
                if (!(inf[e] & 0xffu)) continue;
                if (a.level == a.target) {
                    a.out[pos++] = nug[e];
                    continue;
                }
                const int64_t first = (int64_t)a.prefix[node[e]] - a.off1;
                uint32_t ord = s_order[inf[e] >> 8];
#pragma unroll
                for (int r = 0; r < 8; ++r, ord >>= 3) {
                    const uint32_t j = ord & 7u;
                    if (inf[e] & (1u << j))
                        a.out[pos++] = make_int2(nug[e].x, (int)(first + __popc(oct[e] & ((2u << j) - 1u))));
                }
            }
        }
        __syncthreads();  // s_chunk, s_excl and s_warp are reused by the next chunk
    }
}

__global__ void mark_first_kernel(const int2 *__restrict__ nug, int64_t n, int32_t *__restrict__ info) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        info[i] = (i == 0 || nug[i - 1].x != nug[i].x) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// decode (SPC::SetGeometry)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kChunk) popc_chunk_kernel(const uint8_t *__restrict__ oct, const int64_t *count,
                                                            uint32_t *partials) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t v = i < n ? (uint32_t)__popc(oct[i]) : 0u;
        const uint32_t s = block_sum(v, s_warp);
        if (threadIdx.x == 0) partials[c] = s;
    }
}

// prefix[i] = children of nodes before i, for i in [0, n] (n + 1 entries; the
// count passed covers n + 1 elements, byte n reads as 0).
__global__ void __launch_bounds__(kChunk) popc_prefix_kernel(const uint8_t *__restrict__ oct, int64_t nbytes,
                                                             const int64_t *count, const uint32_t *partials,
                                                             uint32_t *prefix) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t v = i < nbytes ? (uint32_t)__popc(oct[i]) : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < n) prefix[i] = partials[c] + ex;
    }
}

// Level sizes from the prefix table: level 0 = the root; level l+1 has
// prefix[end_l] - prefix[start_l] nodes.  out[0..levels] = counts,
// out[kMaxSpcLevels+1] = number of levels (the leaf level index).
__global__ void level_sizes_kernel(const uint32_t *prefix, int64_t osize, int64_t *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t start = 0, cnt = 1;
    int l = 0;
    out[0] = 1;
    while (start < osize && l < kMaxSpcLevels) {
        const int64_t end = start + cnt;
        const int64_t next = (int64_t)prefix[end < osize ? end : osize] - (int64_t)prefix[start];
        start = end;
        cnt = next;
        ++l;
        out[l] = cnt;
    }
    out[kMaxSpcLevels + 1] = (start == osize) ? l : -1;
}

// Children Morton codes of one level's nodes; codes are staged in the points
// buffer itself (8 bytes per point) and converted to coordinates at the end.
__global__ void nodes_to_morton_kernel(const uint8_t *__restrict__ oct, const uint32_t *__restrict__ prefix,
                                       uint64_t *codes, int64_t start, int64_t cnt) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride) {
        const int64_t node = start + k;
        const uint32_t bits = oct[node];
        const uint64_t m = codes[node];
        int64_t addr = 1 + (int64_t)prefix[node];
        for (int j = 0; j < 8; ++j)
            if (bits & (1u << j)) codes[addr++] = 8ull * m + (uint64_t)j;
    }
}

__global__ void morton_to_points_kernel(uint64_t *codes_then_points, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t m = codes_then_points[i];
        uint32_t x = 0, y = 0, z = 0;
        for (int b = 0; b < 16; ++b) {
            x |= (uint32_t)((m >> (3 * b + 2)) & 1u) << b;
            y |= (uint32_t)((m >> (3 * b + 1)) & 1u) << b;
            z |= (uint32_t)((m >> (3 * b)) & 1u) << b;
        }
        short4 p = make_short4((short)x, (short)y, (short)z, 0);
        reinterpret_cast<short4 *>(codes_then_points)[i] = p;
    }
}

// ---------------------------------------------------------------------------
// build (points -> octree)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    uint64_t m = 0;
    for (int b = 0; b < 16; ++b) {
        m |= (uint64_t)((z >> b) & 1u) << (3 * b);
        m |= (uint64_t)((y >> b) & 1u) << (3 * b + 1);
        m |= (uint64_t)((x >> b) & 1u) << (3 * b + 2);
    }
    return m;
}

__global__ void mark_leaves_kernel(const uint16_t *__restrict__ pts, int64_t n, int level, uint8_t *occ,
                                   int64_t *status) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const uint32_t lim = 1u << level;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
        if (x >= lim || y >= lim || z >= lim) {
            *status = 2;
            continue;
        }
        occ[morton3(x, y, z)] = 1;
    }
}

// Child-occupancy byte of every node of a level from the next level's bytes
// (or leaf occupancy): byte[m] = sum_j [child 8m+j occupied] << j.
__global__ void reduce_level_kernel(const uint8_t *__restrict__ child, int64_t nparents, uint8_t *__restrict__ bytes) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nparents; m += stride) {
        const uint2 c = reinterpret_cast<const uint2 *>(child)[m];  // 8 child entries
        uint32_t b = 0;
        for (int j = 0; j < 4; ++j) {
            if ((c.x >> (8 * j)) & 0xffu) b |= 1u << j;
            if ((c.y >> (8 * j)) & 0xffu) b |= 1u << (j + 4);
        }
        bytes[m] = (uint8_t)b;
    }
}

__global__ void __launch_bounds__(kChunk) nonzero_chunk_kernel(const uint8_t *__restrict__ v, const int64_t *count,
                                                               uint32_t *partials) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && v[i]) ? 1u : 0u;
        const uint32_t s = block_sum(f, s_warp);
        if (threadIdx.x == 0) partials[c] = s;
    }
}

__global__ void __launch_bounds__(kChunk) nonzero_emit_kernel(const uint8_t *__restrict__ v, const int64_t *count,
                                                              const uint32_t *partials, uint8_t *out,
                                                              int64_t out_cap, int64_t *status) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && v[i]) ? 1u : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(f, s_warp, &tot);
        if (f) {
            const int64_t pos = (int64_t)partials[c] + ex;
            if (pos < out_cap)
                out[pos] = v[i];
            else
                *status = 1;
        }
    }
}

// ---------------------------------------------------------------------------
// octree from a field: voxel centres and band selection
// ---------------------------------------------------------------------------
// Centres of voxels [start, start + count) of a 2^level grid in [-1, 1]^3,
// linear index (x * res + y) * res + z.
__global__ void voxel_centres_kernel(int level, int64_t start, int64_t count, float *out) {
    const int64_t res = (int64_t)1 << level;
    const float inv = 2.f / (float)res;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
        const int64_t v = start + k;
        const int64_t x = v / (res * res), y = (v / res) % res, z = v % res;
        out[3 * k] = ((float)x + 0.5f) * inv - 1.f;
        out[3 * k + 1] = ((float)y + 0.5f) * inv - 1.f;
        out[3 * k + 2] = ((float)z + 0.5f) * inv - 1.f;
    }
}

__global__ void __launch_bounds__(kChunk) band_chunk_kernel(const float *__restrict__ d, const int64_t *count,
                                                            float band, uint32_t *partials) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && fabsf(d[i]) <= band) ? 1u : 0u;
        const uint32_t s = block_sum(f, s_warp);
        if (threadIdx.x == 0) partials[c] = s;
    }
}

// Writes the grid coordinates (uint16 x, y, z) of the selected voxels after
// `base` already selected ones.
__global__ void __launch_bounds__(kChunk) band_emit_kernel(const float *__restrict__ d, const int64_t *count,
                                                           float band, const uint32_t *__restrict__ partials,
                                                           int level, int64_t start, uint16_t *out, int64_t base,
                                                           int64_t cap, int64_t *status) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t res = (int64_t)1 << level;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && fabsf(d[i]) <= band) ? 1u : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(f, s_warp, &tot);
        if (!f) continue;
        const int64_t pos = base + (int64_t)partials[c] + ex;
        if (pos >= cap) {
            *status = 1;
            continue;
        }
        const int64_t v = start + i;
        out[3 * pos] = (uint16_t)(v / (res * res));
        out[3 * pos + 1] = (uint16_t)((v / res) % res);
        out[3 * pos + 2] = (uint16_t)(v % res);
    }
}

inline int grid_for(int64_t chunks) {
    const int64_t cap = (int64_t)num_sms() * 2;
    if (chunks < 1) chunks = 1;
    return (int)(chunks < cap ? chunks : cap);
}

inline int grid_elems(int64_t n, int threads = 256) {
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)num_sms() * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace nglod

using namespace nglod;

// Scratch layout of nglod_spc_build: one dense byte array per level l
// (8^l entries, each array starting on a 256-byte boundary so that the
// 8-children reads are aligned), then the chunk partials, then a control
// block of 64 int64.
static int64_t level_array_offset(int l) {
    int64_t t = 0;
    for (int k = 0; k < l; ++k) t += (((int64_t)1 << (3 * k)) + 255) & ~(int64_t)255;
    return t;
}
static int64_t build_dense_bytes(int level) { return level_array_offset(level + 1); }

extern "C" int64_t nglod_spc_build_scratch_bytes(int32_t level) {
    if (level < 1 || level > 9) return -1;
    const int64_t dense = build_dense_bytes(level);
    const int64_t parts = ((int64_t)1 << (3 * level)) / kChunk + 2;
    return dense + ((parts * 4 + 255) & ~(int64_t)255) + 64 * 8;
}

extern "C" int nglod_spc_build(const uint16_t *pts, int64_t n, int32_t level, uint8_t *octree, int64_t octree_cap,
                               int64_t *osize, int32_t *pyramid_host, void *scratch, nglod_stream_t stream) {
    NGLOD_REQUIRE(level >= 1 && level <= 9, NGLOD_ERR_UNSUPPORTED, "octree level=%d outside [1, 9]", level);
    NGLOD_REQUIRE(n >= 1, NGLOD_ERR_INVALID, "n=%lld: an octree needs at least one voxel", (long long)n);
    NGLOD_REQUIRE(pts && octree && osize && pyramid_host && scratch, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(scratch, 256), NGLOD_ERR_ALIGN, "scratch must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t dense = build_dense_bytes(level);
    uint8_t *base = static_cast<uint8_t *>(scratch);
    // level l's dense array starts at off[l]; leaf level last
    std::vector<int64_t> off(level + 1);
    for (int l = 0; l <= level; ++l) off[l] = level_array_offset(l);
    uint32_t *partials = reinterpret_cast<uint32_t *>(base + dense);
    const int64_t parts = ((int64_t)1 << (3 * level)) / kChunk + 2;
    int64_t *ctrl = reinterpret_cast<int64_t *>(base + dense + ((parts * 4 + 255) & ~(int64_t)255));
    NGLOD_TRY(cuda_status(cudaMemsetAsync(base, 0, (size_t)dense, s), "nglod_spc_build memset"));
    NGLOD_TRY(cuda_status(cudaMemsetAsync(ctrl, 0, 64 * sizeof(int64_t), s), "nglod_spc_build memset"));
    mark_leaves_kernel<<<grid_elems(n), 256, 0, s>>>(pts, n, level, base + off[level], ctrl);
    for (int l = level - 1; l >= 0; --l)
        reduce_level_kernel<<<grid_elems((int64_t)1 << (3 * l)), 256, 0, s>>>(base + off[l + 1],
                                                                            (int64_t)1 << (3 * l), base + off[l]);
    NGLOD_TRY(launch_status("nglod_spc_build (levels)"));
    // Compact each level's nonzero bytes in Morton order; counts of levels
    // 0..level (level = occupied leaves) go to ctrl[8 + l].
    int64_t *status = ctrl;
    std::vector<int64_t> counts(level + 1);
    int64_t written = 0;
    for (int l = 0; l <= level; ++l) {
        const int64_t n_l = (int64_t)1 << (3 * l);
        NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl + 2, &n_l, sizeof(int64_t), cudaMemcpyHostToDevice, s),
                              "nglod_spc_build copy"));
        const int64_t chunks = (n_l + kChunk - 1) / kChunk;
        nonzero_chunk_kernel<<<grid_for(chunks), kChunk, 0, s>>>(base + off[l], ctrl + 2, partials);
        scan_chunk_counts_kernel<<<1, kChunk, 0, s>>>(partials, ctrl + 2, ctrl + 8 + l, INT64_MAX, nullptr);
        if (l < level)
            nonzero_emit_kernel<<<grid_for(chunks), kChunk, 0, s>>>(base + off[l], ctrl + 2, partials,
                                                                    octree + written, octree_cap - written, status);
        NGLOD_TRY(launch_status("nglod_spc_build (compact)"));
        NGLOD_TRY(cuda_status(cudaMemcpyAsync(&counts[l], ctrl + 8 + l, sizeof(int64_t), cudaMemcpyDeviceToHost, s),
                              "nglod_spc_build copy"));
        NGLOD_TRY(cuda_status(cudaStreamSynchronize(s), "nglod_spc_build sync"));
        if (l < level) written += counts[l];
        NGLOD_REQUIRE(written <= octree_cap, NGLOD_ERR_CAPACITY, "octree needs more than %lld bytes",
                      (long long)octree_cap);
    }
    int64_t st = 0;
    NGLOD_TRY(cuda_status(cudaMemcpy(&st, status, sizeof(int64_t), cudaMemcpyDeviceToHost), "nglod_spc_build copy"));
    NGLOD_REQUIRE(st != 2, NGLOD_ERR_INVALID, "a voxel coordinate is >= 2^level");
    NGLOD_REQUIRE(st == 0, NGLOD_ERR_CAPACITY, "octree capacity exceeded");
    *osize = written;
    int64_t sum = 0;
    for (int l = 0; l <= level; ++l) {
        pyramid_host[l] = (int32_t)counts[l];
        pyramid_host[(level + 2) + l] = (int32_t)sum;
        sum += counts[l];
    }
    pyramid_host[level + 1] = 0;
    pyramid_host[(level + 2) + level + 1] = (int32_t)sum;
    return NGLOD_OK;
}

extern "C" int nglod_spc_decode(const uint8_t *octree, int64_t osize, int16_t *points, int64_t points_cap,
                                uint32_t *prefix, int32_t *pyramid_host, int32_t *level_out, nglod_stream_t stream) {
    NGLOD_REQUIRE(osize >= 1, NGLOD_ERR_INVALID, "osize=%lld: empty octree", (long long)osize);
    NGLOD_REQUIRE(octree && points && prefix && pyramid_host && level_out, NGLOD_ERR_INVALID,
                  "null pointer argument");
    NGLOD_REQUIRE(aligned(points, 8), NGLOD_ERR_ALIGN, "points must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    // The scan's control block and chunk partials are staged in the points
    // buffer (at least osize + 1 entries of 8 bytes), which is rewritten
    // afterwards.
    const int64_t nelem = osize + 1;
    const int64_t chunks = (nelem + kChunk - 1) / kChunk;
    NGLOD_REQUIRE(points_cap >= osize + 1 && points_cap * 8 >= (chunks + 2) * 4 + 64 * 8 + 8 * (kMaxSpcLevels + 2),
                  NGLOD_ERR_CAPACITY, "points buffer of %lld entries is too small", (long long)points_cap);
    uint8_t *tmp = reinterpret_cast<uint8_t *>(points);
    int64_t *ctrl = reinterpret_cast<int64_t *>(tmp);
    int64_t *sizes = ctrl + 8;
    uint32_t *partials = reinterpret_cast<uint32_t *>(sizes + kMaxSpcLevels + 2);
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl, &nelem, sizeof(int64_t), cudaMemcpyHostToDevice, s), "decode copy"));
    popc_chunk_kernel<<<grid_for(chunks), kChunk, 0, s>>>(octree, ctrl, partials);
    scan_chunk_counts_kernel<<<1, kChunk, 0, s>>>(partials, ctrl, ctrl + 1, INT64_MAX, nullptr);
    popc_prefix_kernel<<<grid_for(chunks), kChunk, 0, s>>>(octree, osize, ctrl, partials, prefix);
    level_sizes_kernel<<<1, 32, 0, s>>>(prefix, osize, sizes);
    NGLOD_TRY(launch_status("nglod_spc_decode (scan)"));
    int64_t hs[kMaxSpcLevels + 2];
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(hs, sizes, sizeof(hs), cudaMemcpyDeviceToHost, s), "decode copy"));
    NGLOD_TRY(cuda_status(cudaStreamSynchronize(s), "decode sync"));
    const int64_t L = hs[kMaxSpcLevels + 1];
    NGLOD_REQUIRE(L >= 1, NGLOD_ERR_INVALID, "octree bytes do not describe a complete tree of <= %d levels",
                  kMaxSpcLevels);
    int64_t psize = 0;
    for (int l = 0; l <= L; ++l) psize += hs[l];
    NGLOD_REQUIRE(psize <= points_cap, NGLOD_ERR_CAPACITY, "octree has %lld points, buffer holds %lld",
                  (long long)psize, (long long)points_cap);
    uint64_t *codes = reinterpret_cast<uint64_t *>(points);
    NGLOD_TRY(cuda_status(cudaMemsetAsync(codes, 0, sizeof(uint64_t), s), "decode memset"));
    int64_t start = 0;
    for (int l = 0; l < L; ++l) {
        nodes_to_morton_kernel<<<grid_elems(hs[l]), 256, 0, s>>>(octree, prefix, codes, start, hs[l]);
        start += hs[l];
    }
    morton_to_points_kernel<<<grid_elems(psize), 256, 0, s>>>(codes, psize);
    NGLOD_TRY(launch_status("nglod_spc_decode (points)"));
    int64_t sum = 0;
    for (int l = 0; l <= L; ++l) {
        pyramid_host[l] = (int32_t)hs[l];
        pyramid_host[(L + 2) + l] = (int32_t)sum;
        sum += hs[l];
    }
    pyramid_host[L + 1] = 0;
    pyramid_host[(L + 2) + L + 1] = (int32_t)sum;
    *level_out = (int32_t)L;
    return NGLOD_OK;
}

extern "C" int nglod_spc_raytrace(const uint8_t *octree, const int16_t *points, const uint32_t *prefix,
                                  const int32_t *pyramid_host, int32_t level, int32_t target_level, const float *org,
                                  const float *dir, int64_t n_rays, int32_t *nuggets_a, int32_t *nuggets_b,
                                  int64_t capacity, uint32_t *info, uint32_t *partials, int64_t *ctrl, int64_t *count,
                                  int32_t *result_buffer, nglod_stream_t stream) {
    NGLOD_REQUIRE(level >= 1 && level < kMaxSpcLevels, NGLOD_ERR_INVALID, "level=%d outside [1, %d)", level,
                  kMaxSpcLevels);
    NGLOD_REQUIRE(target_level >= 0 && target_level <= level, NGLOD_ERR_INVALID,
                  "target_level=%d outside [0, level=%d]", target_level, level);
    // a level's hit count is at most 8 x capacity (eight children per
    // nugget) and the chunk states hold it in 32 bits
    NGLOD_REQUIRE(n_rays >= 0 && n_rays <= capacity && capacity < ((int64_t)1 << 29), NGLOD_ERR_CAPACITY,
                  "n_rays=%lld must not exceed capacity=%lld (< 2^29)", (long long)n_rays, (long long)capacity);
    NGLOD_REQUIRE(pyramid_host && count && result_buffer, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(pyramid_host[level + 1] == 0 && pyramid_host[level + 2] == 0, NGLOD_ERR_INVALID,
                  "bad pyramid table (the reference's 'bad spc table3' check)");
    // Pass l writes level l+1's nuggets to buffer (l+1) % 2; target 0 runs one
    // root-only pass (level 0, writing buffer 1).
    const int passes = target_level == 0 ? 1 : target_level;
    *result_buffer = passes % 2;
    *count = 0;
    if (n_rays == 0) return NGLOD_OK;
    NGLOD_REQUIRE(octree && points && prefix && org && dir && nuggets_a && nuggets_b && info && ctrl,
                  NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(points, 8) && aligned(nuggets_a, 8) && aligned(nuggets_b, 8) && aligned(ctrl, 8),
                  NGLOD_ERR_ALIGN, "points, nuggets and ctrl must be 8-byte aligned");
    NGLOD_REQUIRE(aligned(info, 8), NGLOD_ERR_ALIGN, "info must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    int64_t init[kCtrlCount + 1] = {0, 0, 0, 0, n_rays};
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl, init, sizeof(init), cudaMemcpyHostToDevice, s), "raytrace copy"));
    // tickets and chunk states of every pass start at zero
    const int64_t nstate = state_words(capacity);
    NGLOD_TRY(cuda_status(cudaMemsetAsync(info, 0, (size_t)(kTicketBytes + passes * nstate * 8), s),
                          "raytrace scratch"));
    TraverseArgs a;
    a.octree = octree;
    a.points = reinterpret_cast<const short4 *>(points);
    a.prefix = prefix;
    a.org = org;
    a.dir = dir;
    a.ctrl = ctrl;
    a.capacity = capacity;
    a.target = target_level;
    const int32_t *psum = pyramid_host + (level + 2);
    int2 *buf[2] = {reinterpret_cast<int2 *>(nuggets_a), reinterpret_cast<int2 *>(nuggets_b)};
    unsigned long long *states =
        reinterpret_cast<unsigned long long *>(reinterpret_cast<uint8_t *>(info) + kTicketBytes);
    const int64_t chunks = (capacity + kChunk - 1) / kChunk, cap = (int64_t)num_sms() * 8;
    const int grid = (int)(chunks < cap ? chunks : cap);
    for (int l = 0; l < passes; ++l) {
        a.level = l;
        a.off0 = psum[l];
        a.off1 = psum[l + 1];
        a.in = buf[l % 2];
        a.out = buf[(l + 1) % 2];
        a.state = states + l * nstate;
        a.ticket = info + l;
        traverse_level_kernel<<<grid, kTravThreads, 0, s>>>(a);
    }
    NGLOD_TRY(launch_status("nglod_spc_raytrace"));
    int64_t res[kCtrlCount + kMaxSpcLevels + 1];
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(res, ctrl, sizeof(int64_t) * (kCtrlCount + target_level + 2),
                                          cudaMemcpyDeviceToHost, s),
                          "raytrace copy"));
    NGLOD_TRY(cuda_status(cudaStreamSynchronize(s), "raytrace sync"));
    NGLOD_REQUIRE(res[kCtrlStatus] != kStatusLookback, NGLOD_ERR_CUDA,
                  "spc_raytrace: a chunk's wait for its predecessors gave up");
    NGLOD_REQUIRE(res[kCtrlStatus] == 0, NGLOD_ERR_CAPACITY,
                  "spc_raytrace: more than capacity=%lld nuggets at some level", (long long)capacity);
    *count = res[kCtrlCount + passes];
    return NGLOD_OK;
}

extern "C" int nglod_spc_mark_first(const int32_t *nuggets, int64_t n, int32_t *info, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(nuggets && info, NGLOD_ERR_INVALID, "null pointer argument");
    mark_first_kernel<<<grid_elems(n), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const int2 *>(nuggets), n,
                                                                        info);
    return launch_status("nglod_spc_mark_first");
}

namespace nglod {
struct Mat4 {
    float m[4][4];
};

// a (row vector) times M with the reference's mul4x4 arithmetic
// (spc_math.h:102-110) compiled with default contraction:
// fma(a.w, m3, fma(a.z, m2, fma(a.x, m0, a.y*m1))).
__device__ __forceinline__ float4 row_times(float4 a, const Mat4 &M) {
    float4 r;
    r.x = __fmaf_rn(a.w, M.m[3][0], __fmaf_rn(a.z, M.m[2][0], __fmaf_rn(a.x, M.m[0][0], __fmul_rn(a.y, M.m[1][0]))));
    r.y = __fmaf_rn(a.w, M.m[3][1], __fmaf_rn(a.z, M.m[2][1], __fmaf_rn(a.x, M.m[0][1], __fmul_rn(a.y, M.m[1][1]))));
    r.z = __fmaf_rn(a.w, M.m[3][2], __fmaf_rn(a.z, M.m[2][2], __fmaf_rn(a.x, M.m[0][2], __fmul_rn(a.y, M.m[1][2]))));
    r.w = __fmaf_rn(a.w, M.m[3][3], __fmaf_rn(a.z, M.m[2][3], __fmaf_rn(a.x, M.m[0][3], __fmul_rn(a.y, M.m[1][3]))));
    return r;
}

__global__ void generate_rays_kernel(const Mat4 M, int width, int64_t n, float *org, float *dir) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float px = (float)(uint32_t)(i % width), py = (float)(uint32_t)(i / width);
        const float4 a = row_times(make_float4(0.f, 0.f, 1.f, 0.f), M);
        const float4 b = row_times(make_float4(px, py, 0.f, 1.f), M);
        org[3 * i] = a.x;
        org[3 * i + 1] = a.y;
        org[3 * i + 2] = a.z;
        dir[3 * i] = b.x;
        dir[3 * i + 1] = b.y;
        dir[3 * i + 2] = b.z;
    }
}
}  // namespace nglod

extern "C" int nglod_spc_generate_rays(const float *inv_wvp_host, int32_t width, int32_t height, float *org,
                                       float *dir, nglod_stream_t stream) {
    NGLOD_REQUIRE(width > 0 && height > 0, NGLOD_ERR_INVALID, "image %dx%d is empty", width, height);
    NGLOD_REQUIRE(inv_wvp_host && org && dir, NGLOD_ERR_INVALID, "null pointer argument");
    Mat4 M;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) M.m[r][c] = inv_wvp_host[4 * r + c];
    const int64_t n = (int64_t)width * height;
    generate_rays_kernel<<<grid_elems(n), 256, 0, (cudaStream_t)stream>>>(M, width, n, org, dir);
    return launch_status("nglod_spc_generate_rays");
}

extern "C" int nglod_spc_prefix(const uint8_t *octree, int64_t osize, uint32_t *prefix, uint32_t *partials,
                                int64_t *ctrl, nglod_stream_t stream) {
    NGLOD_REQUIRE(osize >= 0, NGLOD_ERR_INVALID, "osize=%lld is negative", (long long)osize);
    NGLOD_REQUIRE(prefix && partials && ctrl && (octree || osize == 0), NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(ctrl, 8), NGLOD_ERR_ALIGN, "ctrl must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nelem = osize + 1;
    const int64_t chunks = (nelem + kChunk - 1) / kChunk;
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl, &nelem, sizeof(int64_t), cudaMemcpyHostToDevice, s), "prefix copy"));
    popc_chunk_kernel<<<grid_for(chunks), kChunk, 0, s>>>(octree, ctrl, partials);
    scan_chunk_counts_kernel<<<1, kChunk, 0, s>>>(partials, ctrl, ctrl + 1, INT64_MAX, nullptr);
    popc_prefix_kernel<<<grid_for(chunks), kChunk, 0, s>>>(octree, osize, ctrl, partials, prefix);
    return launch_status("nglod_spc_prefix");
}

extern "C" int nglod_voxel_centres(int32_t level, int64_t start, int64_t count, float *out, nglod_stream_t stream) {
    NGLOD_REQUIRE(level >= 1 && level <= 15 && start >= 0 && count >= 0 &&
                      start + count <= ((int64_t)1 << (3 * level)),
                  NGLOD_ERR_INVALID, "voxels [%lld, +%lld) outside the 2^%d grid", (long long)start,
                  (long long)count, level);
    if (count == 0) return NGLOD_OK;
    NGLOD_REQUIRE(out, NGLOD_ERR_INVALID, "null pointer argument");
    voxel_centres_kernel<<<grid_elems(count), 256, 0, (cudaStream_t)stream>>>(level, start, count, out);
    return launch_status("nglod_voxel_centres");
}

extern "C" int nglod_select_band(const float *values, int64_t n, float band, int32_t level, int64_t start,
                                 uint16_t *voxels, int64_t base, int64_t capacity, uint32_t *partials, int64_t *ctrl,
                                 int64_t *selected, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && level >= 1 && level <= 15 && base >= 0 && selected, NGLOD_ERR_INVALID, "bad argument");
    *selected = 0;
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(values && voxels && partials && ctrl, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(ctrl, 8), NGLOD_ERR_ALIGN, "ctrl must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t init[3] = {n, 0, 0};  // count, total, status
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl, init, sizeof(init), cudaMemcpyHostToDevice, s), "band copy"));
    const int grid = grid_for((n + kChunk - 1) / kChunk);
    band_chunk_kernel<<<grid, kChunk, 0, s>>>(values, ctrl, band, partials);
    scan_chunk_counts_kernel<<<1, kChunk, 0, s>>>(partials, ctrl, ctrl + 1, INT64_MAX, nullptr);
    band_emit_kernel<<<grid, kChunk, 0, s>>>(values, ctrl, band, partials, level, start, voxels, base, capacity,
                                             ctrl + 2);
    NGLOD_TRY(launch_status("nglod_select_band"));
    int64_t res[3];
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(res, ctrl, sizeof(res), cudaMemcpyDeviceToHost, s), "band copy"));
    NGLOD_TRY(cuda_status(cudaStreamSynchronize(s), "band sync"));
    NGLOD_REQUIRE(res[2] == 0, NGLOD_ERR_CAPACITY, "more than %lld voxels selected", (long long)(capacity - base));
    *selected = res[1];
    return NGLOD_OK;
}
