/*
 * ORACLE -- test infrastructure only.  Included last by the generated
 * oracle/_ref/ref_gpu.cu.  Launches the DYFOX reference kernels on the GPU
 * exactly as laue/solver.py:74-86 and 107-116 do: grid (Ny * n_e,), block
 * (256,) (backend.py:15), dynamic shared memory 2 * 4 * (Nx + 1) * itemsize
 * (laue/kernels.py:391-393) with the opt-in attribute above 48 KB
 * (kernels.py:372-388).  Returns a cudaError_t.
 */
#include <cuda_runtime.h>

template <class K>
static int ref_gpu_launch(K kernel, int Ny, int n_e, int Nx, size_t item,
                          void *stream, void **args) {
    size_t smem = 2 * 4 * (size_t)(Nx + 1) * item;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            (const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    cudaError_t e = cudaLaunchKernel((const void *)kernel, dim3(Ny * n_e),
                                     dim3(256), args, smem,
                                     (cudaStream_t)stream);
    return (int)e;
}

#define REF_GPU_PARAMS(T) T *Dg_re, T *Dg_im, T s0r, T s0i, T shr, T shi, \
    T sbr, T sbi, T *s_dev, int n_e, T dz, T shift_px, T ds, T dx, int Nz, \
    int Nx, int Ny, T sheet_hw, T fov_hy
#define REF_GPU_ARGV &Dg_re, &Dg_im, &s0r, &s0i, &shr, &shi, &sbr, &sbi, \
    &s_dev, &n_e, &dz, &shift_px, &ds, &dx, &Nz, &Nx, &Ny, &sheet_hw, &fov_hy

#define REF_GPU_ENTRIES(T, SFX)                                              \
extern "C" int ref_gpu_fullfield##SFX(REF_GPU_PARAMS(T), T *H_grid,          \
                                       void *stream) {                       \
    void *args[] = {REF_GPU_ARGV, &H_grid};                                  \
    return ref_gpu_launch(ref_fullfield##SFX::tt3d_fullfield_batch##SFX, Ny, \
                          n_e, Nx, sizeof(T), stream, args);                 \
}                                                                             \
extern "C" int ref_gpu_pristine##SFX(REF_GPU_PARAMS(T), void *stream) {      \
    void *args[] = {REF_GPU_ARGV};                                           \
    return ref_gpu_launch(ref_pristine##SFX::tt3d_pristine_batch##SFX, Ny,   \
                          n_e, Nx, sizeof(T), stream, args);                 \
}                                                                             \
extern "C" int ref_gpu_analytic##SFX(REF_GPU_PARAMS(T), const T *an,          \
                                      void *stream) {                        \
    T a0 = an[0], a1 = an[1], a2 = an[2], a3 = an[3], a4 = an[4], a5 = an[5];\
    T a6 = an[6], a7 = an[7], a8 = an[8], a9 = an[9], a10 = an[10];          \
    T a11 = an[11];                                                           \
    void *args[] = {REF_GPU_ARGV, &a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7,    \
                    &a8, &a9, &a10, &a11};                                   \
    return ref_gpu_launch(ref_analytic##SFX::tt3d_analytic_batch##SFX, Ny,   \
                          n_e, Nx, sizeof(T), stream, args);                 \
}

REF_GPU_ENTRIES(double, _f64)
REF_GPU_ENTRIES(float, _f32)
