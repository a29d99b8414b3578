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

// the same chains on packed FP32 pairs (one fma.rn.f32x2 per two FMAs)
__global__ void fma_chains_x2(float2 *out, int iters, float a, float b) {
    float2 x[8];
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = make_float2((threadIdx.x + k) * 1e-3f, (threadIdx.x + k) * 2e-3f);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = __ffma2_rn(x[k], a2, b2);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k].x + x[k].y;
    if (s == -1.f) out[blockIdx.x * blockDim.x + threadIdx.x] = make_float2(s, s);
}

template <class T>
void launch_chains(int blocks, int threads, cudaStream_t st, T *out, int iters) {
    fma_chains<T><<<blocks, threads, 0, st>>>(out, iters, (T)0.999, (T)1e-6);
}
template <>
void launch_chains<float2>(int blocks, int threads, cudaStream_t st, float2 *out, int iters) {
    fma_chains_x2<<<blocks, threads, 0, st>>>(out, iters, 0.999f, 1e-6f);
}

template <class T>
int probe(double *tflops, int iters, int lanes = 1) {
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
        launch_chains<T>(blocks, threads, c->stream, out, iters);
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
    *tflops = 2.0 * 8.0 * lanes * (double)iters * threads * blocks / (best * 1e-3) / 1e12;
    return 0;
}

}  // namespace

extern "C" {
int p3t_probe_fma_peak(int fp64, double *tflops) {
    if (fp64 == 2) return probe<float2>(tflops, 32768, 2);
    return fp64 ? probe<double>(tflops, 4096) : probe<float>(tflops, 65536);
}
}
