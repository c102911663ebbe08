// FP64 and FP32 pipe throughput probes used by the benchmark for the roofline
// denominators of the FP64 kernels and of the FP32 precision-form kernel (the
// measured peaks cover HBM and bf16 only).  Eight independent
// dependency chains per thread, 8 CTAs per SM.
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

__global__ void k_probe_ffma(float *out, int iters, float a, float b)
{
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fmaf(x[i], a, b);
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// out[0] FFMA instructions/s (best of 3): the FP32 pipe peak of the
// precision-form roofline (one FFMA = two operations); returns 0 or a CUDA
// error code.
extern "C" int vefem_probe_fp32(int device, double *out)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256, iters = 16384;
    float *d = nullptr;
    if ((e = cudaMalloc(&d, sizeof(float) * blocks * threads)) != cudaSuccess) return (int)e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const double ops = 8.0 * iters * (double)blocks * threads;
    double best = 0.0;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(a);
        k_probe_ffma<<<blocks, threads>>>(d, iters, 0.9999999f, 1e-7f);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        const double r = ops / (ms * 1e-3);
        if (r > best) best = r;
    }
    out[0] = best;
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    return (int)e;
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

// ---------------------------------------------------------------------------
// Check of the shared-divisor division (div_r in vefem_physics.cuh) against the
// IEEE division on n pseudo-random operand pairs: random signs and mantissas,
// dividend exponents in [-60, 60], divisor exponents in [-30, 30], and one in
// four divisors drawn from awkward mantissas (all ones, a power of two, one
// ulp above or below one).  Counts bitwise mismatches.
#include "vefem_physics.cuh"

__device__ __forceinline__ uint64_t probe_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double probe_double(uint64_t h, int emin, int espan)
{
    const uint64_t sign = (h >> 63) << 63;
    const int ex = emin + (int)((h >> 52) % (uint64_t)espan);
    const uint64_t mant = h & 0xFFFFFFFFFFFFFULL;
    return __longlong_as_double((long long)(sign | ((uint64_t)(ex + 1023) << 52) | mant));
}

__global__ void k_probe_div(uint64_t n, uint64_t seed, unsigned long long *mism, int *flag,
                            double *example)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t h1 = probe_mix(seed ^ (2 * i)), h2 = probe_mix(seed ^ (2 * i + 1));
        const double x = probe_double(h1, -60, 121);
        double y = probe_double(h2, -30, 61);
        const uint64_t kind = (h2 >> 8) & 15;
        const double ey = __longlong_as_double((long long)(((h2 >> 12) % 61 + 1023 - 30) << 52));
        if (kind == 0) y = ey * 1.9999999999999998;          // all-ones mantissa
        else if (kind == 1) y = ey;                            // power of two
        else if (kind == 2) y = ey * 1.0000000000000002;       // one ulp above
        else if (kind == 3) y = ey * 0.99999999999999989;      // one ulp below
        const double q_ieee = x / y;
        const double q = vefem::div_r(x, y, vefem::recip_for_div(y));
        if (__double_as_longlong(q) != __double_as_longlong(q_ieee)) {
            atomicAdd(mism, 1ULL);
            if (atomicCAS(flag, 0, 1) == 0) {
                example[0] = x;
                example[1] = y;
                example[2] = q;
                example[3] = q_ieee;
            }
        }
    }
}

// returns 0 or a CUDA error code; *mismatches: pairs whose quotients differ;
// example[4]: x, y, div_r result, IEEE result of the first mismatch
extern "C" int vefem_probe_div(int device, unsigned long long n, unsigned long long seed,
                               unsigned long long *mismatches, double *example)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    unsigned long long *dm = nullptr;
    int *df = nullptr;
    double *dx = nullptr;
    if ((e = cudaMalloc(&dm, sizeof(*dm))) != cudaSuccess) return (int)e;
    if ((e = cudaMalloc(&df, sizeof(*df))) != cudaSuccess) return (int)e;
    if ((e = cudaMalloc(&dx, 4 * sizeof(double))) != cudaSuccess) return (int)e;
    cudaMemset(dm, 0, sizeof(*dm));
    cudaMemset(df, 0, sizeof(*df));
    cudaMemset(dx, 0, 4 * sizeof(double));
    k_probe_div<<<sms * 8, 256>>>(n, seed, dm, df, dx);
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, dm, sizeof(*dm), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(example, dx, 4 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dm);
    cudaFree(df);
    cudaFree(dx);
    return (int)e;
}
