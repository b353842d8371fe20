// hc_probe.cu -- the device's FP32 / FP64 fused multiply-add throughput,
// measured with a kernel of independent FMA chains (a measurement aid beside
// the HBM roofline: the stage kernels are arithmetic- and issue-heavy).
#include "hc_internal.h"

#include <cuda_runtime.h>

namespace hc {
namespace {

constexpr int kChains = 8;      // independent FMA chains per thread
constexpr int kIters = 4096;    // FMAs per chain

template <typename T>
__global__ void k_fma(T* sink, T seed) {
    T a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = seed + T(threadIdx.x + c);
    T const b = T(0.999999), d = T(1e-7);
#pragma unroll 16
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], b, d);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c];
    if (s == T(-1)) *sink = s;   // never true; keeps the chains live
}

template <typename T>
int measure(double* tflops) {
    int dev = 0, sms = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    T* sink = nullptr;
    HC_CUDA(cudaMalloc(&sink, sizeof(T)));
    unsigned const blocks = (unsigned)sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma<T><<<blocks, threads>>>(sink, T(1));   // warm-up
    cudaEventRecord(e0);
    int const reps = 5;
    for (int r = 0; r < reps; ++r) k_fma<T><<<blocks, threads>>>(sink, T(r));
    cudaEventRecord(e1);
    cudaError_t const err = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return cuda_fail(err, "FMA probe");
    double const flops = 2.0 * kChains * kIters * (double)blocks * threads * reps;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return HC_OK;
}

}  // namespace
}  // namespace hc

extern "C" int hc_measure_fma(int precision, double* tflops) {
    using namespace hc;
    if (!tflops) return fail(HC_ERR_INVALID, "NULL argument");
    if (precision == HC_F32_FUSED) return measure<float>(tflops);
    if (precision == HC_F64_FUSED || precision == HC_F64_PLAIN) return measure<double>(tflops);
    return fail(HC_ERR_INVALID, "precision");
}
