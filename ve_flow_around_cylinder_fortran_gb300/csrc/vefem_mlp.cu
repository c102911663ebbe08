// Small multilayer perceptron for the learned continuation predictor:
// in -> width (GELU) -> ... -> width (GELU) -> out, trained online with Adam.
//
// Weights are kept as FP32 master copies and used in BF16 (rounded to
// nearest even) in the forward and backward products, with FP32
// accumulation; activations, gradients and the optimiser state are FP32.
// GELU is the erf form, 0.5 x (1 + erf(x / sqrt 2)).  The loss is the mean
// squared error over all outputs.  The products run on the tensor cores
// (mma.sync BF16 with FP32 accumulation; FP32 operands as exact sums of three
// BF16 terms, see k_linear_mma); one training iteration (forward, backward,
// Adam) is captured once in a CUDA graph and replayed.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "vefem.h"
#include "vefem_internal.h"

namespace {

struct Layer {
    int in, out;
    float *W = nullptr, *b = nullptr;          // FP32 master [out][in], [out]
    __nv_bfloat16 *Wb = nullptr;               // BF16 copy used by the products
    float *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;   // Adam moments
    float *gW = nullptr, *gb = nullptr;        // gradients
    float *Z = nullptr, *A = nullptr;          // pre-activation, activation [n][out]
    float *dA = nullptr;                       // gradient w.r.t. A [n][out]
};

// ---- products on the tensor cores: mma.sync m16n8k16, BF16 x BF16 -> FP32
//
// The weights enter as their BF16 copy.  The activations and gradients are
// FP32; each is split exactly into three BF16 terms (x = h + m + l: h the
// nearest BF16, m the nearest BF16 of x - h, l of what is left; 8 + 8 + 8
// significand bits cover FP32's 24), so with the exact BF16 x BF16 products
// and FP32 accumulation a product X W^T is the FP32 product of the FP32
// activations with the BF16 weights, as on the CUDA cores.  For the weight
// gradient dZ^T X both operands are FP32: the six split products whose
// magnitude exceeds 2^-24 of the leading one are summed (h h, h m, m h, h l,
// l h, m m).  No atomics: every output is owned by one CTA, results are the
// same on every run.
//
// The products are small (a few hundred rows by 256) and run once per
// training iteration, so they are latency-bound: a CTA computes one 16 x 8
// output tile, its four warps split K and their partial tiles are added in
// warp order through shared memory.  Fragment layouts of m16n8k16
// (g = lane / 4, t = lane % 4): A registers (g, 2t..2t+1), (g+8, 2t..),
// (g, 2t+8..), (g+8, 2t+8..); B registers (k = 2t..2t+1, n = g),
// (k = 2t+8.., n = g); C (g, 2t..2t+1), (g+8, 2t..2t+1).  Two BF16 per 32-bit
// register, the lower index in the low half.
constexpr int MMA_WARPS = 4;

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 (&p)[3])
{
    p[0] = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p[0]);
    p[1] = __float2bfloat16_rn(r1);
    p[2] = __float2bfloat16_rn(r1 - __bfloat162float(p[1]));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

enum { LIN_FWD = 0, LIN_BWD_X = 1, LIN_BWD_W = 2 };

// Operand element loaders (zero outside the matrix).
//   forward  Y = X W^T:   A(m, k) = X[m][k]   (n x in),  B(k, c) = W[c][k]
//   backward dX = dZ W:   A(m, k) = dZ[m][k]  (n x out), B(k, c) = W[k][c]
//   weights  gW = dZ^T X: A(m, k) = dZ[k][m]  (out x n), B(k, c) = X[k][c], and
//                         column c = in the constant 1 (its output is gb)
template <int MODE>
__device__ __forceinline__ float load_a(const float *__restrict__ A, int M, int K, int lda, int m, int k)
{
    if (m >= M || k >= K) return 0.0f;
    return MODE == LIN_BWD_W ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
}

template <int MODE>
__global__ void __launch_bounds__(MMA_WARPS * 32)
k_linear_mma(int M, int N, int K, const float *__restrict__ A, int lda,
             const __nv_bfloat16 *__restrict__ Wb, const float *__restrict__ Bf, int ldb,
             const float *__restrict__ bias, float *__restrict__ out0, float *__restrict__ out1,
             float *__restrict__ out2, int ldo, int gelu)
{
    __shared__ float s_part[MMA_WARPS - 1][32][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * 16, n0 = blockIdx.x * 8;
    const int ksteps = (K + 15) / 16;
    const int per = (ksteps + MMA_WARPS - 1) / MMA_WARPS;
    const int ks1 = min(ksteps, (warp + 1) * per);
    const int c = n0 + g;                  // the B column this thread loads
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 2
    for (int ks = warp * per; ks < ks1; ks++) {
        const int k0 = ks * 16;
        // A fragments of the three split terms
        uint32_t af[3][4];
        {
            const int rows[4] = {m0 + g, m0 + g + 8, m0 + g, m0 + g + 8};
            const int cols[4] = {k0 + 2 * t, k0 + 2 * t, k0 + 2 * t + 8, k0 + 2 * t + 8};
#pragma unroll
            for (int r = 0; r < 4; r++) {
                __nv_bfloat16 lo[3], hi[3];
                split3(load_a<MODE>(A, M, K, lda, rows[r], cols[r]), lo);
                split3(load_a<MODE>(A, M, K, lda, rows[r], cols[r] + 1), hi);
#pragma unroll
                for (int q = 0; q < 3; q++) af[q][r] = pack2(lo[q], hi[q]);
            }
        }
        const int ks_[4] = {k0 + 2 * t, k0 + 2 * t + 1, k0 + 2 * t + 8, k0 + 2 * t + 9};
        if (MODE != LIN_BWD_W) {
            __nv_bfloat16 w[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int k = ks_[u];
                const bool in = c < N && k < K;
                w[u] = in ? (MODE == LIN_FWD ? Wb[(size_t)c * ldb + k] : Wb[(size_t)k * ldb + c])
                          : __float2bfloat16_rn(0.0f);
            }
            const uint32_t b0 = pack2(w[0], w[1]), b1 = pack2(w[2], w[3]);
            // small terms first
            mma_bf16(acc, af[2], b0, b1);
            mma_bf16(acc, af[1], b0, b1);
            mma_bf16(acc, af[0], b0, b1);
        } else {
            __nv_bfloat16 x[4][3];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int k = ks_[u];
                float v = 0.0f;
                if (k < K && c < N) v = c < N - 1 ? Bf[(size_t)k * ldb + c] : 1.0f;
                split3(v, x[u]);
            }
            uint32_t bf[3][2];
#pragma unroll
            for (int q = 0; q < 3; q++) {
                bf[q][0] = pack2(x[0][q], x[1][q]);
                bf[q][1] = pack2(x[2][q], x[3][q]);
            }
            mma_bf16(acc, af[1], bf[1][0], bf[1][1]);
            mma_bf16(acc, af[2], bf[0][0], bf[0][1]);
            mma_bf16(acc, af[0], bf[2][0], bf[2][1]);
            mma_bf16(acc, af[1], bf[0][0], bf[0][1]);
            mma_bf16(acc, af[0], bf[1][0], bf[1][1]);
            mma_bf16(acc, af[0], bf[0][0], bf[0][1]);
        }
    }
    // partial tiles of warps 1..3 added to warp 0's, in warp order
    if (warp > 0) {
#pragma unroll
        for (int u = 0; u < 4; u++) s_part[warp - 1][lane][u] = acc[u];
    }
    __syncthreads();
    if (warp != 0) return;
#pragma unroll
    for (int w = 0; w < MMA_WARPS - 1; w++)
#pragma unroll
        for (int u = 0; u < 4; u++) acc[u] += s_part[w][lane][u];
    // epilogue
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int m = m0 + g + (u >= 2 ? 8 : 0);
        const int cc = n0 + 2 * t + (u & 1);
        if (m >= M || cc >= N) continue;
        const float v = acc[u];
        if (MODE == LIN_FWD) {
            const float z = v + bias[cc];
            out0[(size_t)m * ldo + cc] = z;
            out1[(size_t)m * ldo + cc] = gelu ? 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)) : z;
        } else if (MODE == LIN_BWD_X) {
            out0[(size_t)m * ldo + cc] = v;
        } else {
            if (cc < N - 1) out0[(size_t)m * ldo + cc] = v;
            else out2[m] = v;
        }
    }
}

// dZ = dA * gelu'(Z) (in place into dA when gelu)
__global__ void k_gelu_bwd(int count, const float *__restrict__ Z, float *__restrict__ dA)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float z = Z[i];
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    dA[i] = dA[i] * (cdf + z * pdf);
}

dim3 mma_grid(int M, int N)
{
    return dim3((unsigned)((N + 7) / 8), (unsigned)((M + 15) / 16));
}

// MSE loss and its gradient: dY = 2 (Y - T) / (n out), *loss = mean (Y - T)^2.
// One block: each thread sums its strided share in order, then a fixed tree in
// shared memory -- the same bits on every run (no atomics).
constexpr int MSE_THREADS = 1024;
__global__ void __launch_bounds__(MSE_THREADS) k_mse(int count, const float *__restrict__ Y,
                                                     const float *__restrict__ T,
                                                     float *__restrict__ dY, float *__restrict__ loss)
{
    __shared__ float red[MSE_THREADS];
    float acc = 0.0f;
    for (int i = threadIdx.x; i < count; i += MSE_THREADS) {
        const float d = Y[i] - T[i];
        dY[i] = 2.0f * d / (float)count;
        acc += d * d;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = MSE_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)count;
}

// Adam on the FP32 masters, then the BF16 copy; t is read from device memory
__global__ void k_adam(int count, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, __nv_bfloat16 *pb, float lr,
                       const int *__restrict__ step)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float t = (float)(*step);
    const float mi = b1 * m[i] + (1.0f - b1) * g[i];
    const float vi = b2 * v[i] + (1.0f - b2) * g[i] * g[i];
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, t));
    const float vh = vi / (1.0f - powf(b2, t));
    const float np = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = np;
    if (pb) pb[i] = __float2bfloat16_rn(np);
}

__global__ void k_to_bf16(int count, const float *__restrict__ p, __nv_bfloat16 *pb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) pb[i] = __float2bfloat16_rn(p[i]);
}

__global__ void k_step_inc(int *step, float *loss)
{
    *step += 1;
    *loss = 0.0f;
}

}  // namespace


struct vefem_mlp {
    int device = 0;
    int in = 0, width = 0, out = 0, hidden = 0;
    std::vector<Layer> L;
    int cap = 0;                  // rows the activation buffers hold
    float *X = nullptr, *T = nullptr, *loss = nullptr;
    int *step = nullptr;
    cudaStream_t s = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_n = -1;
    float graph_lr = 0.0f;
    std::string err;
};

namespace {

int mlp_fail(vefem_mlp *m, int code, const std::string &msg)
{
    if (m)
        m->err = msg;
    else
        vefem::set_global_error(msg);
    return code;
}

#define MCK(call)                                                                   \
    do {                                                                            \
        cudaError_t _e = (call);                                                    \
        if (_e != cudaSuccess)                                                      \
            return mlp_fail(m, VEFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

int64_t nparams(const vefem_mlp *m)
{
    int64_t n = 0;
    for (const Layer &l : m->L) n += (int64_t)l.in * l.out + l.out;
    return n;
}

int ensure_rows(vefem_mlp *m, int n)
{
    if (n <= m->cap) return VEFEM_OK;
    for (Layer &l : m->L) {
        cudaFree(l.Z);
        cudaFree(l.A);
        cudaFree(l.dA);
        MCK(cudaMalloc(&l.Z, sizeof(float) * n * l.out));
        MCK(cudaMalloc(&l.A, sizeof(float) * n * l.out));
        MCK(cudaMalloc(&l.dA, sizeof(float) * n * l.out));
    }
    cudaFree(m->X);
    cudaFree(m->T);
    MCK(cudaMalloc(&m->X, sizeof(float) * n * m->in));
    MCK(cudaMalloc(&m->T, sizeof(float) * n * m->out));
    m->cap = n;
    if (m->graph) {
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    return VEFEM_OK;
}

void launch_forward(vefem_mlp *m, int n)
{
    const float *x = m->X;
    for (size_t i = 0; i < m->L.size(); i++) {
        Layer &l = m->L[i];
        // Y[n][out] = X[n][in] W^T + b (GELU but on the last layer); Z keeps the pre-activation
        k_linear_mma<LIN_FWD><<<mma_grid(n, l.out), MMA_WARPS * 32, 0, m->s>>>(
            n, l.out, l.in, x, l.in, l.Wb, nullptr, l.in, l.b, l.Z, l.A, nullptr, l.out,
            i + 1 < m->L.size() ? 1 : 0);
        x = l.A;
    }
}

void launch_backward(vefem_mlp *m, int n)
{
    // dA of the output layer holds dLoss/dY (from k_mse)
    for (int i = (int)m->L.size() - 1; i >= 0; i--) {
        Layer &l = m->L[i];
        if (i + 1 < (int)m->L.size())
            k_gelu_bwd<<<(n * l.out + 255) / 256, 256, 0, m->s>>>(n * l.out, l.Z, l.dA);
        const float *xin = i == 0 ? m->X : m->L[i - 1].A;
        // gW[out][in] = dZ^T X and gb[out] = dZ^T 1 (the extra column)
        k_linear_mma<LIN_BWD_W><<<mma_grid(l.out, l.in + 1), MMA_WARPS * 32, 0, m->s>>>(
            l.out, l.in + 1, n, l.dA, l.out, nullptr, xin, l.in, nullptr, l.gW, nullptr, l.gb,
            l.in, 0);
        if (i > 0) {
            // dX[n][in] = dZ[n][out] W[out][in]
            k_linear_mma<LIN_BWD_X><<<mma_grid(n, l.in), MMA_WARPS * 32, 0, m->s>>>(
                n, l.in, l.out, l.dA, l.out, l.Wb, nullptr, l.in, nullptr, m->L[i - 1].dA,
                nullptr, nullptr, l.in, 0);
        }
    }
}

void launch_loss(vefem_mlp *m, int n)
{
    Layer &o = m->L.back();
    const int count = n * o.out;
    k_mse<<<1, MSE_THREADS, 0, m->s>>>(count, o.A, m->T, o.dA, m->loss);
}

void launch_adam(vefem_mlp *m, float lr)
{
    for (Layer &l : m->L) {
        const int cw = l.in * l.out;
        k_adam<<<(cw + 255) / 256, 256, 0, m->s>>>(cw, l.W, l.gW, l.mW, l.vW, l.Wb, lr, m->step);
        k_adam<<<(l.out + 255) / 256, 256, 0, m->s>>>(l.out, l.b, l.gb, l.mb, l.vb, nullptr, lr,
                                                       m->step);
    }
}

}  // namespace

namespace {

int mlp_init(vefem_mlp *m, uint64_t seed)
{
    const int hidden_layers = m->hidden;
    MCK(cudaSetDevice(m->device));
    MCK(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking));
    // Kaiming-uniform-like init from a 64-bit LCG (deterministic for a seed)
    uint64_t st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&st]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(st >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int i = 0; i <= hidden_layers; i++) {
        Layer l;
        l.in = i == 0 ? m->in : m->width;
        l.out = i == hidden_layers ? m->out : m->width;
        m->L.push_back(l);
    }
    for (Layer &l : m->L) {
        const size_t nw = (size_t)l.in * l.out;
        std::vector<float> w(nw), b(l.out, 0.0f);
        const double bound = std::sqrt(1.0 / l.in);
        for (size_t k = 0; k < nw; k++) w[k] = (float)((2.0 * uni() - 1.0) * bound);
        float **f[] = {&l.W, &l.mW, &l.vW, &l.gW};
        for (float **p : f) MCK(cudaMalloc(p, sizeof(float) * nw));
        float **g[] = {&l.b, &l.mb, &l.vb, &l.gb};
        for (float **p : g) MCK(cudaMalloc(p, sizeof(float) * l.out));
        MCK(cudaMalloc(&l.Wb, sizeof(__nv_bfloat16) * nw));
        MCK(cudaMemcpy(l.W, w.data(), sizeof(float) * nw, cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(l.b, b.data(), sizeof(float) * l.out, cudaMemcpyHostToDevice));
        MCK(cudaMemset(l.mW, 0, sizeof(float) * nw));
        MCK(cudaMemset(l.vW, 0, sizeof(float) * nw));
        MCK(cudaMemset(l.mb, 0, sizeof(float) * l.out));
        MCK(cudaMemset(l.vb, 0, sizeof(float) * l.out));
        k_to_bf16<<<(int)((nw + 255) / 256), 256, 0, m->s>>>((int)nw, l.W, l.Wb);
    }
    MCK(cudaMalloc(&m->loss, sizeof(float)));
    MCK(cudaMalloc(&m->step, sizeof(int)));
    MCK(cudaMemset(m->step, 0, sizeof(int)));
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

}  // namespace

extern "C" int vefem_mlp_create(int in_dim, int width, int out_dim, int hidden_layers,
                                uint64_t seed, int device, vefem_mlp **out)
{
    if (!out || in_dim <= 0 || width <= 0 || out_dim <= 0 || hidden_layers <= 0 || device < 0 ||
        (int64_t)in_dim * width > (1 << 28) || (int64_t)width * out_dim > (1 << 28))
        return mlp_fail(nullptr, VEFEM_ERR_ARG, "vefem_mlp_create: bad arguments");
    *out = nullptr;
    vefem_mlp *m = new vefem_mlp();
    m->device = device;
    m->in = in_dim;
    m->width = width;
    m->out = out_dim;
    m->hidden = hidden_layers;
    if (int rc = mlp_init(m, seed)) {
        vefem::set_global_error("vefem_mlp_create: " + m->err);
        vefem_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return VEFEM_OK;
}

extern "C" int vefem_mlp_reset_optimizer(vefem_mlp *m)
{
    if (!m) return mlp_fail(nullptr, VEFEM_ERR_ARG, "NULL network");
    MCK(cudaSetDevice(m->device));
    for (Layer &l : m->L) {
        const size_t nw = (size_t)l.in * l.out;
        MCK(cudaMemsetAsync(l.mW, 0, sizeof(float) * nw, m->s));
        MCK(cudaMemsetAsync(l.vW, 0, sizeof(float) * nw, m->s));
        MCK(cudaMemsetAsync(l.mb, 0, sizeof(float) * l.out, m->s));
        MCK(cudaMemsetAsync(l.vb, 0, sizeof(float) * l.out, m->s));
    }
    MCK(cudaMemsetAsync(m->step, 0, sizeof(int), m->s));
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

extern "C" int64_t vefem_mlp_num_params(const vefem_mlp *m) { return m ? nparams(m) : -1; }

// parameters as one FP32 array: for each layer W [out][in] then b [out]
extern "C" int vefem_mlp_set_params(vefem_mlp *m, const float *p, int64_t n)
{
    if (!m || !p || n != nparams(m)) return mlp_fail(m, VEFEM_ERR_ARG, "parameter count");
    MCK(cudaSetDevice(m->device));
    int64_t o = 0;
    for (Layer &l : m->L) {
        const size_t nw = (size_t)l.in * l.out;
        MCK(cudaMemcpyAsync(l.W, p + o, sizeof(float) * nw, cudaMemcpyHostToDevice, m->s));
        o += nw;
        MCK(cudaMemcpyAsync(l.b, p + o, sizeof(float) * l.out, cudaMemcpyHostToDevice, m->s));
        o += l.out;
        k_to_bf16<<<(int)((nw + 255) / 256), 256, 0, m->s>>>((int)nw, l.W, l.Wb);
    }
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

extern "C" int vefem_mlp_get_params(const vefem_mlp *mc, float *p, int64_t n)
{
    vefem_mlp *m = const_cast<vefem_mlp *>(mc);
    if (!m || !p || n != nparams(m)) return mlp_fail(m, VEFEM_ERR_ARG, "parameter count");
    MCK(cudaSetDevice(m->device));
    int64_t o = 0;
    for (Layer &l : m->L) {
        const size_t nw = (size_t)l.in * l.out;
        MCK(cudaMemcpyAsync(p + o, l.W, sizeof(float) * nw, cudaMemcpyDeviceToHost, m->s));
        o += nw;
        MCK(cudaMemcpyAsync(p + o, l.b, sizeof(float) * l.out, cudaMemcpyDeviceToHost, m->s));
        o += l.out;
    }
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

extern "C" int vefem_mlp_forward(vefem_mlp *m, const float *X, int n, float *Y)
{
    if (!m || !X || !Y || n <= 0) return mlp_fail(m, VEFEM_ERR_ARG, "bad arguments");
    MCK(cudaSetDevice(m->device));
    if (int rc = ensure_rows(m, n)) return rc;
    MCK(cudaMemcpyAsync(m->X, X, sizeof(float) * n * m->in, cudaMemcpyHostToDevice, m->s));
    launch_forward(m, n);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(Y, m->L.back().A, sizeof(float) * n * m->out, cudaMemcpyDeviceToHost, m->s));
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

// loss and the gradient w.r.t. all parameters (layout of vefem_mlp_get_params)
extern "C" int vefem_mlp_loss_grad(vefem_mlp *m, const float *X, const float *T, int n,
                                   float *loss, float *grad)
{
    if (!m || !X || !T || !loss || !grad || n <= 0) return mlp_fail(m, VEFEM_ERR_ARG, "bad arguments");
    MCK(cudaSetDevice(m->device));
    if (int rc = ensure_rows(m, n)) return rc;
    MCK(cudaMemcpyAsync(m->X, X, sizeof(float) * n * m->in, cudaMemcpyHostToDevice, m->s));
    MCK(cudaMemcpyAsync(m->T, T, sizeof(float) * n * m->out, cudaMemcpyHostToDevice, m->s));
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->s));
    launch_forward(m, n);
    launch_loss(m, n);
    launch_backward(m, n);
    MCK(cudaGetLastError());
    int64_t o = 0;
    for (Layer &l : m->L) {
        const size_t nw = (size_t)l.in * l.out;
        MCK(cudaMemcpyAsync(grad + o, l.gW, sizeof(float) * nw, cudaMemcpyDeviceToHost, m->s));
        o += nw;
        MCK(cudaMemcpyAsync(grad + o, l.gb, sizeof(float) * l.out, cudaMemcpyDeviceToHost, m->s));
        o += l.out;
    }
    MCK(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->s));
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

// iters full-batch Adam iterations on (X, T); one iteration is a CUDA graph
extern "C" int vefem_mlp_train(vefem_mlp *m, const float *X, const float *T, int n, int iters,
                               float lr, float *final_loss)
{
    if (!m || !X || !T || n <= 0 || iters < 0) return mlp_fail(m, VEFEM_ERR_ARG, "bad arguments");
    MCK(cudaSetDevice(m->device));
    if (int rc = ensure_rows(m, n)) return rc;
    MCK(cudaMemcpyAsync(m->X, X, sizeof(float) * n * m->in, cudaMemcpyHostToDevice, m->s));
    MCK(cudaMemcpyAsync(m->T, T, sizeof(float) * n * m->out, cudaMemcpyHostToDevice, m->s));
    if (!m->graph || m->graph_n != n || m->graph_lr != lr) {
        if (m->graph) cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
        cudaGraph_t g;
        MCK(cudaStreamBeginCapture(m->s, cudaStreamCaptureModeThreadLocal));
        k_step_inc<<<1, 1, 0, m->s>>>(m->step, m->loss);
        launch_forward(m, n);
        launch_loss(m, n);
        launch_backward(m, n);
        launch_adam(m, lr);
        MCK(cudaStreamEndCapture(m->s, &g));
        MCK(cudaGraphInstantiate(&m->graph, g, 0));
        cudaGraphDestroy(g);
        m->graph_n = n;
        m->graph_lr = lr;
    }
    for (int i = 0; i < iters; i++) MCK(cudaGraphLaunch(m->graph, m->s));
    if (final_loss) {
        MCK(cudaMemcpyAsync(final_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->s));
    }
    MCK(cudaStreamSynchronize(m->s));
    return VEFEM_OK;
}

extern "C" int vefem_mlp_destroy(vefem_mlp *m)
{
    if (!m) return VEFEM_OK;
    cudaSetDevice(m->device);
    if (m->s) cudaStreamSynchronize(m->s);
    if (m->graph) cudaGraphExecDestroy(m->graph);
    for (Layer &l : m->L) {
        void *p[] = {l.W, l.b, l.Wb, l.mW, l.vW, l.mb, l.vb, l.gW, l.gb, l.Z, l.A, l.dA};
        for (void *q : p)
            if (q) cudaFree(q);
    }
    void *p[] = {m->X, m->T, m->loss, m->step};
    for (void *q : p)
        if (q) cudaFree(q);
    if (m->s) cudaStreamDestroy(m->s);
    delete m;
    return VEFEM_OK;
}

extern "C" const char *vefem_mlp_last_error(const vefem_mlp *m) { return m ? m->err.c_str() : ""; }
