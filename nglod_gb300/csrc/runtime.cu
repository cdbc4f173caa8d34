// Library-wide runtime pieces: version string, per-thread error message,
// cached device properties.
#include <stdarg.h>
#include <stdio.h>

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

}  // namespace nglod

extern "C" const char *nglod_version(void) { return "nglod_gb300 0.1 (sm_103a)"; }

extern "C" const char *nglod_last_error(void) { return nglod::g_last_error; }
