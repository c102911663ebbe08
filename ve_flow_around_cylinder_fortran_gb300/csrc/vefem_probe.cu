// FP64 pipe throughput probe used by the benchmark for the roofline
// denominator of the FP64 kernels (the measured peaks cover HBM and
// bf16 only).  Eight independent dependency chains per thread, 8 CTAs per SM.
#include <cuda_runtime.h>
#include <stdint.h>

__global__ void k_probe_dfma(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_dadd(double *out, int iters, double a)
{
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = x[i] + a;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_dmul(double *out, int iters, double a)
{
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i + 1.0;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = x[i] * a;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// out[0] DFMA instructions/s, out[1] DADD/s, out[2] DMUL/s (best of 3 each);
// returns 0 or a CUDA error code.
extern "C" int vefem_probe_fp64(int device, double *out)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double *d = nullptr;
    if ((e = cudaMalloc(&d, sizeof(double) * blocks * threads)) != cudaSuccess) return (int)e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const double ops = 8.0 * iters * (double)blocks * threads;
    for (int kind = 0; kind < 3; kind++) {
        double best = 0.0;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(a);
            if (kind == 0) k_probe_dfma<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
            if (kind == 1) k_probe_dadd<<<blocks, threads>>>(d, iters, 1e-7);
            if (kind == 2) k_probe_dmul<<<blocks, threads>>>(d, iters, 0.9999999);
            cudaEventRecord(b);
            cudaEventSynchronize(b);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, a, b);
            const double r = ops / (ms * 1e-3);
            if (r > best) best = r;
        }
        out[kind] = best;
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    return (int)e;
}
