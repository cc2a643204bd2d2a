// probe.cu -- FP32 / FP64 fused multiply-add issue rate of the device, used as the
// denominator of the compute roofline (the integrand is CUDA-core bound).
#include <cuda_runtime.h>

#include "g3l_gpu.h"

namespace {

__global__ void fma32_probe(float *out, int iters, float a, float b)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void fma64_probe(double *out, int iters, double a, double b)
{
    double x[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = fma(x[k], a, b);
    out[blockIdx.x * blockDim.x + threadIdx.x] = x[0] + x[1] + x[2] + x[3];
}

}  // namespace

extern "C" int g3l_probe_peaks(int device, cudaStream_t s, double *t32, double *t64)
{
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device)) return G3L_ERR_CUDA;
    const int blocks = nsm * 8, threads = 256;
    void *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * blocks * threads)) return G3L_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best32 = 1e30f, best64 = 1e30f, ms;
    const int it32 = 20000, it64 = 2000;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, s);
        fma32_probe<<<blocks, threads, 0, s>>>((float *)buf, it32, 0.999f, 1e-3f);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best32) best32 = ms;
        cudaEventRecord(e0, s);
        fma64_probe<<<blocks, threads, 0, s>>>((double *)buf, it64, 0.999, 1e-3);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best64) best64 = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (err != cudaSuccess) return G3L_ERR_CUDA;
    *t32 = 2.0 * 8 * it32 * (double)blocks * threads / best32 / 1e9;
    *t64 = 2.0 * 4 * it64 * (double)blocks * threads / best64 / 1e9;
    return G3L_OK;
}
