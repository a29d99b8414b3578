// FMA throughput microbenchmarks: the FP32 and FP64 roofline denominators of
// the soft and hard kernels (the measured-peak file covers only HBM and BF16).
#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"

namespace {

template <class T>
__global__ void fma_chains(T *out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == (T)-1) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <class T>
int probe(double *tflops, int iters) {
    p3t::Context *c = p3t::ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int threads = 256, blocks = sms * 8;
    T *out = nullptr;
    int r = p3t::cuda_status(cudaMalloc(&out, sizeof(T) * threads * blocks));
    if (r) return r;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0, c->stream);
        fma_chains<T><<<blocks, threads, 0, c->stream>>>(out, iters, (T)0.999, (T)1e-6);
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    r = p3t::cuda_status(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (r) return r;
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (best * 1e-3) / 1e12;
    return 0;
}

}  // namespace

extern "C" {
int p3t_probe_fma_peak(int fp64, double *tflops) {
    return fp64 ? probe<double>(tflops, 4096) : probe<float>(tflops, 65536);
}
}
