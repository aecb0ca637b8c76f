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

// Per-kernel CUDA events of the last timed Laue solve on this thread.
static thread_local bool g_timing = false;
static thread_local bool g_events_made = false;
static thread_local unsigned g_marked = 0;
static thread_local cudaEvent_t g_events[kLaueMarks];

void laue_mark(int slot, cudaStream_t stream) {
    if (!g_timing || slot < 0 || slot >= kLaueMarks) return;
    if (slot == 0) g_marked = 0;
    if (cudaEventRecord(g_events[slot], stream) == cudaSuccess)
        g_marked |= 1u << slot;
}

}  // namespace dyfox

extern "C" int dyfox_kernel_timing(int on) {
    using namespace dyfox;
    set_error("");
    if (on && !g_events_made) {
        for (int i = 0; i < kLaueMarks; ++i) {
            cudaError_t e = cudaEventCreate(&g_events[i]);
            if (e != cudaSuccess) return cuda_status(e, "cudaEventCreate");
        }
        g_events_made = true;
    }
    g_timing = on != 0;
    g_marked = 0;
    return DYFOX_OK;
}

extern "C" int dyfox_laue_kernel_ms(float ms[3]) {
    using namespace dyfox;
    set_error("");
    const unsigned all = (1u << kLaueMarks) - 1;
    if (!ms || !g_events_made || g_marked != all) {
        set_error("no timed dyfox_laue_solve on this thread: call "
                  "dyfox_kernel_timing(1) before the solve");
        return DYFOX_EINVAL;
    }
    cudaError_t e = cudaEventSynchronize(g_events[kLaueMarks - 1]);
    if (e != cudaSuccess) return cuda_status(e, "cudaEventSynchronize");
    for (int i = 0; i + 1 < kLaueMarks; ++i) {
        e = cudaEventElapsedTime(&ms[i], g_events[i], g_events[i + 1]);
        if (e != cudaSuccess) return cuda_status(e, "cudaEventElapsedTime");
    }
    return DYFOX_OK;
}

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
