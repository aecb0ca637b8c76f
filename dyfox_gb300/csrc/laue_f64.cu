// Double-precision instantiations of the register-resident Laue march.
#include "laue_march.cuh"

namespace dyfox {

const int kCplF64[] = {4, 5, 6, 7, 8};
const int kNumCplF64 = 5;

#define DYFOX_E64(CPL, HT)                                                   \
    case (CPL) * 4 + (HT):                                                   \
        return {launch_march<double, CPL, HT, false>,                        \
                attr_march<double, CPL, HT, false>};

MarchEntry march_entry_f64(int cpl, int ht) {
    switch (cpl * 4 + ht) {
        DYFOX_E64(4, 0) DYFOX_E64(4, 1) DYFOX_E64(4, 3)
        DYFOX_E64(5, 0) DYFOX_E64(5, 1) DYFOX_E64(5, 3)
        DYFOX_E64(6, 0) DYFOX_E64(6, 1) DYFOX_E64(6, 3)
        DYFOX_E64(7, 0) DYFOX_E64(7, 1) DYFOX_E64(7, 3)
        DYFOX_E64(8, 0) DYFOX_E64(8, 1) DYFOX_E64(8, 3)
    default:
        return {nullptr, nullptr};
    }
}

}  // namespace dyfox
