// Packed-pair (two deviation parameters per thread) instantiations of the
// compensated single-precision Laue march.
#include "laue_pair.cuh"

namespace dyfox {

#define DYFOX_P32(CPL, HT)                                                   \
    case (CPL) * 4 + (HT):                                                   \
        return {launch_pair<CPL, HT>, attr_pair<CPL, HT>};

MarchEntry march_entry_f32_pair(int cpl, int ht) {
    switch (cpl * 4 + ht) {
        DYFOX_P32(3, 0) DYFOX_P32(3, 1) DYFOX_P32(3, 2)
        DYFOX_P32(5, 0) DYFOX_P32(5, 1) DYFOX_P32(5, 2)
        DYFOX_P32(7, 0) DYFOX_P32(7, 1) DYFOX_P32(7, 2)
    default:
        return {nullptr, nullptr};
    }
}

}  // namespace dyfox
