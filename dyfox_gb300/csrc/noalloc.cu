// dyfox_laue_solve_noalloc: the Laue solve for callers that cannot allocate
// device memory when they solve.
//
// Some callers of this library cannot call cudaMalloc, or any allocator, at
// the point where they run a march: a real-time acquisition or
// reconstruction loop that reserves its device memory once at start-up and
// must never fail or stall on an allocation mid-run; a plugin host that
// forbids allocations after initialisation; a plain C or Fortran caller
// that links this library without PyTorch, CuPy or any other device
// allocator.  This entry point gives them the solve without a workspace: the
// scratch lives in one fixed-size array in the library's own device memory.
//
// The array is DYFOX_NOALLOC_SCRATCH_BYTES (32 MiB).  Every GPU that loads
// the library holds it until the process exits.  Its memory is reserved
// when the CUDA module of this file is loaded on a device.  Under CUDA's
// default lazy module loading that is the first call of this entry point on
// that device (its cudaGetSymbolAddress below), so that first call can
// still fail for lack of device memory: a caller that must never meet an
// allocation failure mid-run makes one call during its start-up.  Under
// eager loading (CUDA_MODULE_LOADING=EAGER) every process that loads the
// library holds the array from the start, used or not.  Problems whose
// workspace (dyfox_laue_workspace_bytes) is larger are rejected with
// DYFOX_ENOMEM.  Every call shares the array and the array keeps the last
// call's contents; the solve overwrites every scratch byte it reads
// (per-angle tables, pivots, staged phase) before reading it, so nothing has
// to start at zero.  Calls whose work overlaps on the GPU (concurrent calls
// on different streams, or from different host threads) race on the array:
// serialise them.  The array's address is looked up once per device and
// kept; cudaDeviceReset unloads the module, so after a reset in the same
// process this entry point must not be called again.
#include <mutex>

#include "common.cuh"

namespace dyfox {

static __device__ __align__(256) unsigned char
    g_noalloc_scratch[DYFOX_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[kMaxDevices];

// The array's device address on the current device.  The first call on a
// device resolves it (cudaGetSymbolAddress) with that device current.
static int noalloc_scratch(void **ptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d above the %d supported", dev, kMaxDevices);
        return DYFOX_ENOSYS;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = p;
    }
    *ptr = g_noalloc_ptr[dev];
    return DYFOX_OK;
}

}  // namespace dyfox

extern "C" int dyfox_laue_solve_noalloc(const dyfox_laue_desc *d,
                                        const double *s_dev,
                                        const void *h_grid,
                                        const double *seg_table, void *out,
                                        void *stream) {
    dyfox::set_error("");
    const size_t need = dyfox_laue_workspace_bytes(d);
    if (need > DYFOX_NOALLOC_SCRATCH_BYTES) {
        dyfox::set_error("this problem needs %zu bytes of scratch; the fixed "
                         "array of dyfox_laue_solve_noalloc holds %zu: use "
                         "dyfox_laue_solve with a workspace",
                         need, (size_t)DYFOX_NOALLOC_SCRATCH_BYTES);
        return DYFOX_ENOMEM;
    }
    void *scratch = nullptr;
    int st = dyfox::noalloc_scratch(&scratch);
    if (st) return st;
    // An invalid descriptor (need == 0) is reported by dyfox_laue_solve.
    return dyfox_laue_solve(d, s_dev, h_grid, seg_table, out, scratch,
                            DYFOX_NOALLOC_SCRATCH_BYTES, stream);
}
