// Mixed-precision Bragg GMRES kernels of batches (one CTA per
// system of many instances); see bragg_solve.cuh.
#include "bragg_solve.cuh"

namespace dyfox {

cudaError_t bragg_batch_smem32(int cpl, size_t smem, int threads) {
    switch (cpl) {
    case 1: return set_smem_t<1, true>(smem, threads);
    case 2: return set_smem_t<2, true>(smem, threads);
    case 4: return set_smem_t<4, true>(smem, threads);
    case 8: return set_smem_t<8, true>(smem, threads);
    default: return set_smem_t<16, true>(smem, threads);
    }
}

cudaError_t bragg_batch_launch32(const BraggArgs *insts, const int2 *systems,
                                 int n_sys, int threads, int cpl, size_t smem,
                                 cudaStream_t stream) {
#define DYFOX_BB(C) \
    launch_bragg_batch_t<C, true>(insts, systems, n_sys, threads, smem, stream)
    switch (cpl) {
    case 1: return DYFOX_BB(1);
    case 2: return DYFOX_BB(2);
    case 4: return DYFOX_BB(4);
    case 8: return DYFOX_BB(8);
    default: return DYFOX_BB(16);
    }
#undef DYFOX_BB
}

}  // namespace dyfox
