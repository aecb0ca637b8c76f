// Shared definitions of the dyfox_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/dyfox_gb300.h"

namespace dyfox {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.283185307179586;           // 2 * np.pi
// 2 pi split for an accurate double-precision Cody-Waite reduction.
constexpr double kTwoPiHi = 6.28318530717958623200e+00;
constexpr double kTwoPiLo = 2.44929359829470635445e-16;
constexpr double kInvTwoPi = 0.15915494309189533577;

// Segment-table layout (DYFOX_SEG_STRIDE doubles per segment).
enum SegField {
    SEG_CX = 0, SEG_CY, SEG_CZ,          // core (segment midpoint)
    SEG_XI = 3,                          // unit line direction (3)
    SEG_E1 = 6,                          // unit edge direction (3)
    SEG_E2 = 9,                          // xi x e1 (3)
    SEG_CATAN = 12,                      // g.e1 b_perp + g.xi b_screw
    SEG_GE1 = 13, SEG_GE2 = 14, SEG_BPERP = 15,
    // Single-precision form, pixel units (d -> d / dx):
    SEG_KX = 16,                         // coefficient of d1 d2 / r2c
    SEG_KL = 17,                         // coefficient of ln r2c
    SEG_KQ = 18,                         // coefficient of (d1^2-d2^2)/r2c
    SEG_HCONST = 19,                     // K_l ln(dx^2), kept in double
    SEG_C1 = 20,                         // b_perp / (2 pi)
    SEG_A2PX = 21,                       // (a_core / dx)^2
    SEG_SLOPE1 = 22, SEG_SLOPE2 = 23     // d(d1)/dx, d(d2)/dx along a row
};

template <typename R> struct RT;
template <> struct RT<double> { using R2 = double2; };
template <> struct RT<float> { using R2 = float2; };

// Set by each entry point on failure; read by dyfox_last_error().
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *where);
// Adds n to the launch counter read by dyfox_launch_count().
void count_launch(unsigned n);
// The counter's value, and setting it back (launches recorded into a CUDA
// graph during stream capture run only when the graph is replayed).
unsigned long long launch_count_value();
void launch_count_restore(unsigned long long v);

inline int div_up(int a, int b) { return (a + b - 1) / b; }

// Kernel timing of dyfox_laue_solve (dyfox_kernel_timing): marks 0..3 are
// recorded on the solve's stream before the prologue, after it, after the
// phase staging and after the march, when timing is on for the thread.
constexpr int kLaueMarks = 4;
void laue_mark(int slot, cudaStream_t stream);

}  // namespace dyfox
