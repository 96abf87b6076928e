// Library core: version, per-thread error messages, device properties.
#include <stdarg.h>
#include <stdio.h>

#include "common.cuh"

namespace vs {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return VS_ERR_CUDA;
    }
    return VS_OK;
}

int sm_count() {
    static thread_local int cached_dev = -1, cached = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (dev != cached_dev) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cached_dev = dev;
        cached = n;
    }
    return cached;
}

}  // namespace vs

extern "C" const char *vs_version(void) { return "vissat-gb300 0.1.0 (sm_103a)"; }

extern "C" const char *vs_last_error(void) { return vs::g_last_error; }
