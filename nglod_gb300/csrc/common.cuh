// Shared helpers of the nglod_gb300 CUDA library: status reporting, launch
// geometry, and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nglod_gb300.h"

namespace nglod {

// Records a printf-style message as this host thread's last error.
void set_error(const char *fmt, ...);

// NGLOD_OK if e == cudaSuccess, else records "<where>: <cuda message>" and
// returns NGLOD_ERR_CUDA.
int cuda_status(cudaError_t e, const char *where);

// Launch status of the last kernel launch on this thread.
inline int launch_status(const char *where) { return cuda_status(cudaGetLastError(), where); }

// Multiprocessor count of the current device (cached per device).
int num_sms();

// Bound of the tensor-core wait of the float32 query kernel (dense.cu);
// nglod_debug_mma_wait_polls sets it with the BF16 kernels' bound.
void set_f32tc_wait_polls(uint32_t polls);

inline bool aligned(const void *p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

// Host-memory queries: points [n][3] and results [n] in host memory.  When
// both are pinned and mapped, one kernel launch reads and writes them over
// the host link directly.  Otherwise they go in chunks through a device
// staging area of kHostStages buffers; chunk i runs H2D -> kernel -> D2H on
// stage i % kHostStages, whose stream is the caller's (stage 0) or one of
// the library's helper streams of the current device, forked from and
// joined back into the caller's stream, so that the copies of one chunk
// overlap the kernels of the others.
constexpr int kHostStages = 3;
int64_t host_stage_bytes(int64_t chunk);
// launch(x_dev, m, out_dev, stream) queues one chunk's kernel.
using HostChunkLaunch = int (*)(const void *ctx, const float *x, int64_t m, float *out, cudaStream_t s);
int host_query_pipeline(const float *x_host, int64_t n, float *out_host, int64_t chunk, void *scratch,
                        cudaStream_t stream, HostChunkLaunch launch, const void *ctx);

}  // namespace nglod

#define NGLOD_REQUIRE(cond, code, ...)        \
    do {                                      \
        if (!(cond)) {                        \
            ::nglod::set_error(__VA_ARGS__);  \
            return (code);                    \
        }                                     \
    } while (0)

#define NGLOD_TRY(expr)            \
    do {                           \
        int _st = (expr);          \
        if (_st != NGLOD_OK)       \
            return _st;            \
    } while (0)
