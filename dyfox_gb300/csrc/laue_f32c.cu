// Single-precision compensated (Fast2Sum) instantiations of the register-resident Laue march.
#include "laue_march.cuh"

namespace dyfox {

#define DYFOX_E32(CPL, HT)                                                   \
    case (CPL) * 4 + (HT):                                                   \
        return {launch_march<float, CPL, HT, true>,                          \
                attr_march<float, CPL, HT, true>};

MarchEntry march_entry_f32_comp(int cpl, int ht) {
    switch (cpl * 4 + ht) {
        DYFOX_E32(5, 0) DYFOX_E32(5, 1) DYFOX_E32(5, 2) DYFOX_E32(5, 3)
        DYFOX_E32(7, 0) DYFOX_E32(7, 1) DYFOX_E32(7, 2) DYFOX_E32(7, 3)
        DYFOX_E32(9, 0) DYFOX_E32(9, 1) DYFOX_E32(9, 2) DYFOX_E32(9, 3)
        DYFOX_E32(11, 0) DYFOX_E32(11, 1) DYFOX_E32(11, 2) DYFOX_E32(11, 3)
        DYFOX_E32(13, 0) DYFOX_E32(13, 1) DYFOX_E32(13, 2) DYFOX_E32(13, 3)
    default:
        return {nullptr, nullptr};
    }
}

}  // namespace dyfox
