// Chunk scans: stream compaction for variable-length outputs.  A chunk is
// 1024 consecutive elements handled by one 1024-thread block iteration; a
// first pass reduces each chunk to a count, scan_chunk_counts_kernel (one
// block) turns the counts into exclusive chunk offsets and their total, and a
// last pass rescans each chunk to place its survivors.
#pragma once

#include "common.cuh"

namespace nglod {

constexpr int kChunk = 1024;

// ---------------------------------------------------------------------------
// block scan helpers (blockDim.x == kChunk)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        s_warp[lane] = wi - w;  // exclusive prefix of warp totals
        if (lane == 31) s_warp[32] = wi;
    }
    __syncthreads();
    const uint32_t r = s_warp[warp] + x - v;
    *total = s_warp[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *s_warp) {
    uint32_t t;
    block_exclusive_scan(v, s_warp, &t);
    return t;
}

// Pass 2: exclusive scan of `nchunks` chunk counts in place, in one block.
// The total goes to *total_out (and, if over `capacity`, raises the status).
static __global__ void __launch_bounds__(kChunk) scan_chunk_counts_kernel(uint32_t *partials, const int64_t *count_in,
                                                                   int64_t *total_out, int64_t capacity,
                                                                   int64_t *status) {
    __shared__ uint32_t s_warp[33];
    const int64_t count = *count_in;
    // A raised status (an earlier level overflowed) or a count beyond the
    // capacity the partials were sized for: nothing may be read or written.
    if (status && (*status != 0 || count > capacity)) {
        if (threadIdx.x == 0) {
            *status = 1;
            *total_out = 0;
        }
        return;
    }
    const int64_t nchunks = (count + kChunk - 1) / kChunk;
    uint64_t carry = 0;
    for (int64_t base = 0; base < nchunks; base += kChunk) {
        const int64_t i = base + threadIdx.x;
        const uint32_t v = i < nchunks ? partials[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < nchunks) partials[i] = (uint32_t)(carry + ex);
        carry += tot;
    }
    if (threadIdx.x == 0) {
        *total_out = (int64_t)carry;
        if ((int64_t)carry > capacity && status) *status = 1;
    }
}

}  // namespace nglod
