// Throughput probes used by bench.py to put FP64-bound kernels on a roofline:
// FP64 / FP32 FMA issue rate and device-to-device copy bandwidth, measured on
// the GPU the benchmark runs on.  Built as a separate library
// (lib/libsfem_probe.so); nothing in libsmearfem_gpu.so depends on it.
#include <cuda_runtime.h>
#include <stdint.h>

#define PROBE_API extern "C" __attribute__((visibility("default")))

namespace {

constexpr int CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma(T *out, int iters, T a, T b) {
    T x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == (T)-12345.678) out[threadIdx.x] = s;  // keeps the chains live
}

// FP64 tensor-core rate: independent chains of mma.sync m8n8k4 (one warp
// instruction = 8 x 8 x 4 FMAs = 512 FLOP) on register fragments.
constexpr int MMA_CHAINS = 8;

__global__ void __launch_bounds__(256) k_dmma(double *out, int iters, double a0, double b0) {
    const double a = a0 * (double)(threadIdx.x + 1), b = b0;
    double c[MMA_CHAINS][2];
#pragma unroll
    for (int k = 0; k < MMA_CHAINS; ++k) c[k][0] = c[k][1] = 1e-3 * (double)k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int k = 0; k < MMA_CHAINS; ++k)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                             : "+d"(c[k][0]), "+d"(c[k][1])
                             : "d"(a), "d"(b));
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < MMA_CHAINS; ++k) s += c[k][0] + c[k][1];
    if (s == -12345.678) out[threadIdx.x] = s;  // keeps the chains live
}

__global__ void k_copy(const double2 *__restrict__ a, double2 *__restrict__ b, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) b[i] = a[i];
}

template <typename T>
int fma_peak(int device, double *tflops) {
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, device);
    T *out = nullptr;
    if (cudaMalloc(&out, 256 * sizeof(T)) != cudaSuccess) return 1;
    const int blocks = p.multiProcessorCount * 8, iters = sizeof(T) == 8 ? 256 : 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma<T><<<blocks, 256>>>(out, iters, (T)0.999999, (T)1e-7);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        k_fma<T><<<blocks, 256>>>(out, iters, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const double flops = 2.0 * CHAINS * 16.0 * iters * (double)blocks * 256.0;
    *tflops = flops / (best * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

PROBE_API int sfem_probe_fp64_tflops(int device, double *tflops) { return fma_peak<double>(device, tflops); }

// FP64 tensor-core (DMMA) throughput, best of 5.
PROBE_API int sfem_probe_dmma_tflops(int device, double *tflops) {
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, device);
    double *out = nullptr;
    if (cudaMalloc(&out, 256 * sizeof(double)) != cudaSuccess) return 1;
    const int blocks = p.multiProcessorCount * 8, iters = 64;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dmma<<<blocks, 256>>>(out, iters, 0.999999, 1e-7);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        k_dmma<<<blocks, 256>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const double warps = (double)blocks * 256.0 / 32.0;
    const double flops = 512.0 * MMA_CHAINS * 16.0 * iters * warps;
    *tflops = flops / (best * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
PROBE_API int sfem_probe_fp32_tflops(int device, double *tflops) { return fma_peak<float>(device, tflops); }

// Read+write bytes per second of a device copy of `bytes` bytes (best of 5).
PROBE_API int sfem_probe_copy_gbs(int device, size_t bytes, double *gbs) {
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    const size_t n = bytes / sizeof(double2);
    double2 *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, n * sizeof(double2)) != cudaSuccess) return 1;
    if (cudaMalloc(&b, n * sizeof(double2)) != cudaSuccess) {
        cudaFree(a);
        return 1;
    }
    cudaMemset(a, 0, n * sizeof(double2));
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, device);
    const int blocks = p.multiProcessorCount * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_copy<<<blocks, 256>>>(a, b, n);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        k_copy<<<blocks, 256>>>(a, b, n);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    *gbs = 2.0 * n * sizeof(double2) / (best * 1e-3) / 1e9;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
