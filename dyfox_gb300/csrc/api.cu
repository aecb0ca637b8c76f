// Status reporting of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "common.cuh"

namespace dyfox {

static thread_local char g_error[512];

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof g_error, fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return DYFOX_OK;
    set_error("%s: %s", where, cudaGetErrorString(e));
    return DYFOX_ECUDA;
}

}  // namespace dyfox

extern "C" const char *dyfox_status_string(int status) {
    switch (status) {
    case DYFOX_OK: return "ok";
    case DYFOX_EINVAL: return "invalid argument";
    case DYFOX_ENOMEM: return "workspace too small";
    case DYFOX_ESMEM: return "shared memory above the device limit";
    case DYFOX_EMAXITER: return "iteration cap reached";
    case DYFOX_ENAN: return "non-finite value";
    case DYFOX_ECUDA: return "CUDA error";
    case DYFOX_ENOSYS: return "configuration not supported";
    default: return "unknown status";
    }
}

extern "C" const char *dyfox_last_error(void) { return dyfox::g_error; }

extern "C" int dyfox_abi_version(void) { return DYFOX_ABI_VERSION; }
