// Diagnostics: the FMA-pipe throughput probe (roofline denominator of the
// arithmetic-bound kernels) and the library's kernel-launch counter.
#include <atomic>

#include "common.cuh"
#include "volterra.cuh"

namespace dyfox {

std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned n) { g_launches += n; }
unsigned long long launch_count_value() { return g_launches.load(); }
void launch_count_restore(unsigned long long v) { g_launches.store(v); }

// Eight independent FMA chains per thread, `iters` rounds each.
template <typename R>
__global__ void fma_probe_kernel(R *out, int iters, R a, R b) {
    R v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (R)(threadIdx.x + i);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = v[i] * a + b;
    }
    R s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += v[i];
    if (s == (R)-1.2345) out[0] = s;   // keeps the chains live
}

template <typename R>
static int run_probe(int iters, double *tflops, cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e) return cuda_status(e, "probe device query");
    R *out = nullptr;
    cudaEvent_t t0, t1;
    // The probe is a diagnostic outside the hot path: it owns its events
    // and one scalar of device memory for the duration of the call.
    if ((e = cudaMallocAsync((void **)&out, sizeof(R), stream)))
        return cuda_status(e, "probe alloc");
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    const int blocks = sms * 8, threads = 256;
    fma_probe_kernel<R><<<blocks, threads, 0, stream>>>(out, 64, (R)0.999, (R)1e-3);
    cudaEventRecord(t0, stream);
    fma_probe_kernel<R><<<blocks, threads, 0, stream>>>(out, iters, (R)0.999, (R)1e-3);
    cudaEventRecord(t1, stream);
    e = cudaEventSynchronize(t1);
    float ms = 0;
    if (!e) e = cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFreeAsync(out, stream);
    if (e) return cuda_status(e, "probe timing");
    double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return DYFOX_OK;
}

// The single-precision building blocks of the fused Volterra phase beside
// CUDA's correctly rounded operations, elementwise (dyfox_arith_probe).
__global__ void arith_probe_kernel(int op, const float *__restrict__ a,
                                   const float *__restrict__ b, void *out,
                                   int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    switch (op) {
    case 0: ((float *)out)[i] = rcp_nr(a[i]); break;
    case 1: ((float *)out)[i] = __frcp_rn(a[i]); break;
    case 2: ((float *)out)[i] = div_nr(a[i], b[i]); break;
    case 3: ((float *)out)[i] = __fdiv_rn(a[i], b[i]); break;
    case 4: ((double *)out)[i] = widen_f32(a[i]); break;
    default: ((double *)out)[i] = (double)a[i]; break;
    }
}

// The double-precision building blocks of the FP64 Volterra field beside
// CUDA's, elementwise (dyfox_arith_probe64).
__global__ void arith_probe64_kernel(int op, const double *__restrict__ a,
                                     const double *__restrict__ b,
                                     double *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    switch (op) {
    case 0: out[i] = atan2_d(a[i], b[i]); break;
    case 1: out[i] = atan2(a[i], b[i]); break;
    case 2: out[i] = log_d(a[i]); break;
    case 3: out[i] = log(a[i]); break;
    case 4: out[i] = rcp_d(a[i]); break;
    default: out[i] = __drcp_rn(a[i]); break;
    }
}

// The FP64 segment sum (seg_sum64, constant 0) of each group of m floats
// (dyfox_seg_sum_probe).
__global__ void seg_sum_probe_kernel(const float *__restrict__ terms, int m,
                                     double *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *t = terms + (size_t)i * m;
    out[i] = seg_sum64(m, 0.0, [&](int s) { return t[s]; });
}

}  // namespace dyfox

extern "C" int dyfox_seg_sum_probe(const float *terms, int m, double *out,
                                   int n, void *stream) {
    dyfox::set_error("");
    if (m < 0 || n < 0 || (n > 0 && (!out || (m > 0 && !terms)))) {
        dyfox::set_error("bad arguments to dyfox_seg_sum_probe");
        return DYFOX_EINVAL;
    }
    if (n == 0) return DYFOX_OK;
    dyfox::seg_sum_probe_kernel<<<(n + 255) / 256, 256, 0,
                                  (cudaStream_t)stream>>>(terms, m, out, n);
    dyfox::count_launch(1);
    return dyfox::cuda_status(cudaGetLastError(), "seg_sum_probe");
}

extern "C" int dyfox_arith_probe64(int op, const double *a, const double *b,
                                   double *out, int n, void *stream) {
    dyfox::set_error("");
    if (op < 0 || op > 5 || n < 0 || (n > 0 && (!a || !out)) ||
        ((op == 0 || op == 1) && n > 0 && !b)) {
        dyfox::set_error("bad arguments to dyfox_arith_probe64");
        return DYFOX_EINVAL;
    }
    if (n == 0) return DYFOX_OK;
    dyfox::arith_probe64_kernel<<<(n + 255) / 256, 256, 0,
                                  (cudaStream_t)stream>>>(op, a, b, out, n);
    dyfox::count_launch(1);
    return dyfox::cuda_status(cudaGetLastError(), "arith_probe64");
}

extern "C" int dyfox_arith_probe(int op, const float *a, const float *b,
                                 void *out, int n, void *stream) {
    dyfox::set_error("");
    if (op < 0 || op > 5 || n < 0 || (n > 0 && (!a || !out)) ||
        ((op == 2 || op == 3) && n > 0 && !b)) {
        dyfox::set_error("bad arguments to dyfox_arith_probe");
        return DYFOX_EINVAL;
    }
    if (n == 0) return DYFOX_OK;
    dyfox::arith_probe_kernel<<<(n + 255) / 256, 256, 0,
                                (cudaStream_t)stream>>>(op, a, b, out, n);
    dyfox::count_launch(1);
    return dyfox::cuda_status(cudaGetLastError(), "arith_probe");
}

extern "C" int dyfox_pipe_peak(int precision, int iters, double *tflops,
                               void *stream) {
    dyfox::set_error("");
    if (!tflops || iters < 1) {
        dyfox::set_error("bad arguments to dyfox_pipe_peak");
        return DYFOX_EINVAL;
    }
    if (precision == DYFOX_FP64)
        return dyfox::run_probe<double>(iters, tflops, (cudaStream_t)stream);
    return dyfox::run_probe<float>(iters, tflops, (cudaStream_t)stream);
}

extern "C" unsigned long long dyfox_launch_count(void) {
    return dyfox::g_launches.load();
}
