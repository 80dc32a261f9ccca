// Host runtime shared by every entry point: error reporting and device info.
#include <cstdarg>
#include <cstdio>

#include "gb_common.cuh"

namespace gb {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int num_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    return sms > 0 ? sms : 1;
}

}  // namespace gb

extern "C" const char *gb_last_error_string(void) { return gb::g_err; }

extern "C" int gb_version(void) { return 10000; }
