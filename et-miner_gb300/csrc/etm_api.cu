// Library-wide entry points: version, last error, device properties.
#include <stdarg.h>

#include "etm_common.cuh"

namespace etm {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

const char* last_error() { return g_err; }

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

}  // namespace etm

extern "C" int etm_version(void) { return 1; }
extern "C" const char* etm_last_error(void) { return etm::last_error(); }
extern "C" int etm_device_sm_count(void) { return etm::sm_count(); }
