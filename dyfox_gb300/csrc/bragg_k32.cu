// Mixed-precision Bragg GMRES kernels of single solve calls
// (and the parity-check operators); see bragg_solve.cuh.
#include "bragg_solve.cuh"

namespace dyfox {

cudaError_t bragg_launch_solve32(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, cudaStream_t stream) {
    switch (cpl) {
    case 1: return launch_gmres<1, true>(a, threads, smem, grid, stream);
    case 2: return launch_gmres<2, true>(a, threads, smem, grid, stream);
    case 4: return launch_gmres<4, true>(a, threads, smem, grid, stream);
    case 8: return launch_gmres<8, true>(a, threads, smem, grid, stream);
    default: return launch_gmres<16, true>(a, threads, smem, grid, stream);
    }
}

cudaError_t bragg_launch_apply32(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, int mode,
                                 const double2 *d0, const double2 *dg,
                                 double2 *out, cudaStream_t stream) {
#define DYFOX_APPLY(C) \
    launch_apply<C, true>(a, threads, smem, grid, mode, d0, dg, out, stream)
    switch (cpl) {
    case 1: return DYFOX_APPLY(1);
    case 2: return DYFOX_APPLY(2);
    case 4: return DYFOX_APPLY(4);
    case 8: return DYFOX_APPLY(8);
    default: return DYFOX_APPLY(16);
    }
#undef DYFOX_APPLY
}

}  // namespace dyfox
