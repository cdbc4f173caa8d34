// Library-wide runtime pieces: version string, per-thread error message,
// cached device properties.
#include <stdarg.h>
#include <stdio.h>

#include <mutex>

#include "common.cuh"

namespace nglod {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return NGLOD_OK;
    set_error("%s: %s", where, cudaGetErrorString(e));
    return NGLOD_ERR_CUDA;
}

int num_sms() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (cache[dev] == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// Helper streams of one device (created on first use, kept for the life of
// the process) and the fork / join events of the pipeline.  The mutex keeps
// one pipeline's event record / wait pairs from interleaving with another's.
struct HostStages {
    std::mutex mu;
    bool ready = false;
    cudaStream_t aux[kHostStages - 1] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kHostStages - 1] = {};
};
static HostStages g_stages[64];

int64_t host_stage_bytes(int64_t chunk) {
    const int64_t xs = (chunk * 12 + 255) & ~(int64_t)255, os = (chunk * 4 + 255) & ~(int64_t)255;
    return kHostStages * (xs + os);
}

// The device address of host memory the GPU reads and writes directly
// (pinned and mapped: cudaHostAlloc, cudaHostRegister), else null.
static void *mapped_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int host_query_pipeline(const float *x_host, int64_t n, float *out_host, int64_t chunk, void *scratch,
                        cudaStream_t stream, HostChunkLaunch launch, const void *ctx) {
    NGLOD_REQUIRE(n >= 0 && chunk >= 1, NGLOD_ERR_INVALID, "n=%lld, chunk=%lld", (long long)n, (long long)chunk);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x_host && out_host && scratch, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(scratch, 256), NGLOD_ERR_ALIGN, "scratch must be 256-byte aligned");
    // Pinned, mapped host buffers: the kernel reads the points and writes
    // the results over the host link itself, in one launch, with no staging
    // copies.
    const float *x_map = static_cast<const float *>(mapped_host(x_host));
    float *out_map = static_cast<float *>(mapped_host(out_host));
    if (x_map && out_map) return launch(ctx, x_map, n, out_map, stream);
    int dev = 0;
    NGLOD_TRY(cuda_status(cudaGetDevice(&dev), "host query: device"));
    NGLOD_REQUIRE(dev >= 0 && dev < 64, NGLOD_ERR_UNSUPPORTED, "device %d", dev);
    HostStages &hs = g_stages[dev];
    std::lock_guard<std::mutex> g(hs.mu);
    if (!hs.ready) {
        for (int i = 0; i < kHostStages - 1; ++i) {
            NGLOD_TRY(cuda_status(cudaStreamCreateWithFlags(&hs.aux[i], cudaStreamNonBlocking), "host query: stream"));
            NGLOD_TRY(cuda_status(cudaEventCreateWithFlags(&hs.join[i], cudaEventDisableTiming), "host query: event"));
        }
        NGLOD_TRY(cuda_status(cudaEventCreateWithFlags(&hs.fork, cudaEventDisableTiming), "host query: event"));
        hs.ready = true;
    }
    cudaStream_t st[kHostStages];
    st[0] = stream;
    for (int i = 1; i < kHostStages; ++i) st[i] = hs.aux[i - 1];
    const int64_t xs = (chunk * 12 + 255) & ~(int64_t)255, os = (chunk * 4 + 255) & ~(int64_t)255;
    char *base = static_cast<char *>(scratch);
    NGLOD_TRY(cuda_status(cudaEventRecord(hs.fork, stream), "host query: fork"));
    for (int i = 1; i < kHostStages; ++i)
        NGLOD_TRY(cuda_status(cudaStreamWaitEvent(st[i], hs.fork, 0), "host query: fork"));
    int status = NGLOD_OK;
    int64_t k = 0;
    for (int64_t c = 0; c < n && status == NGLOD_OK; c += chunk, ++k) {
        const int64_t m = n - c < chunk ? n - c : chunk;
        const int b = (int)(k % kHostStages);
        float *xd = reinterpret_cast<float *>(base + b * (xs + os));
        float *od = reinterpret_cast<float *>(base + b * (xs + os) + xs);
        status = cuda_status(cudaMemcpyAsync(xd, x_host + 3 * c, (size_t)m * 12, cudaMemcpyHostToDevice, st[b]),
                             "host query: copy in");
        if (status == NGLOD_OK) status = launch(ctx, xd, m, od, st[b]);
        if (status == NGLOD_OK)
            status = cuda_status(cudaMemcpyAsync(out_host + c, od, (size_t)m * 4, cudaMemcpyDeviceToHost, st[b]),
                                 "host query: copy out");
    }
    // join every helper stream back into the caller's, also after an error
    for (int i = 1; i < kHostStages; ++i) {
        const int e1 = cuda_status(cudaEventRecord(hs.join[i - 1], st[i]), "host query: join");
        const int e2 = e1 == NGLOD_OK ? cuda_status(cudaStreamWaitEvent(stream, hs.join[i - 1], 0), "host query: join")
                                      : e1;
        if (status == NGLOD_OK) status = e2;
    }
    return status;
}

}  // namespace nglod

extern "C" int64_t nglod_host_query_scratch_bytes(int64_t chunk) { return chunk >= 1 ? nglod::host_stage_bytes(chunk) : -1; }

extern "C" const char *nglod_version(void) { return "nglod_gb300 0.1 (sm_103a)"; }

extern "C" const char *nglod_last_error(void) { return nglod::g_last_error; }
