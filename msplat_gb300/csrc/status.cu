// Status strings, last-error detail and device queries for the C ABI.
#include <stdarg.h>

#include <atomic>

#include "common.cuh"

namespace msplat {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

static std::atomic<unsigned long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (cached[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 1;
    }
    return cached[dev];
}

}  // namespace msplat

extern "C" const char *msplat_status_string(int status) {
    switch (status) {
        case MSPLAT_OK: return "ok";
        case MSPLAT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case MSPLAT_ERR_WORKSPACE: return "workspace too small";
        case MSPLAT_ERR_LAUNCH: return "kernel launch failed";
        case MSPLAT_ERR_CAPACITY: return "capacity exceeded";
        case MSPLAT_ERR_UNSUPPORTED: return "unsupported configuration";
        case MSPLAT_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown status";
    }
}

extern "C" const char *msplat_last_error(void) { return msplat::g_last_error; }

extern "C" const char *msplat_version(void) { return "0.1.0"; }

extern "C" unsigned long long msplat_kernel_launches(void) {
    return msplat::g_launches.load(std::memory_order_relaxed);
}
