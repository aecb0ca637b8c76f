/*
 * ORACLE -- test infrastructure only.
 *
 * Lets the DYFOX reference kernel text (laue/kernels.py:48-352, written
 * into oracle/_ref/ by oracle/make_ref.py) compile as plain C++ for the CPU.
 * Each kernel is run with blockDim.x == 1: its strided column loops then
 * cover every column with a single thread, so __syncthreads() has nothing
 * to order and is a no-op.  Blocks run in parallel under OpenMP, so the
 * block index and the dynamic shared-memory buffer are thread-local.
 */
#pragma once
#include <cmath>
#include <cstddef>

struct RefDim3 { int x, y, z; };
extern thread_local RefDim3 blockIdx;
extern thread_local RefDim3 threadIdx;
extern thread_local RefDim3 blockDim;

#define __global__
#define __shared__ thread_local
/* Backing store of each kernel's `extern __shared__ T smem[]` (renamed per
 * kernel by make_ref.py), one per thread: four rows of Nx + 1 amplitudes,
 * double-buffered, for Nx up to 8191.  C linkage, like the declaration. */
#define REF_SMEM_DEF(T, NAME) extern "C" { thread_local T NAME[2 * 4 * 8192]; }
#define __syncthreads() ((void)0)

using std::atan2; using std::cos; using std::exp; using std::fabs;
using std::floor; using std::log; using std::sin; using std::sqrt;
