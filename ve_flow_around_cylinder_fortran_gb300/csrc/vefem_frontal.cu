// Panel-frontal elimination of the bordered Newton Jacobian on the device: the
// Newton and continuation drivers' linear solver, in place of the MUMPS
// factorisation and solve behind KSPSolve (Petsc_mod.F90:850).
//
// The symbolic phase (element panels, pivots and fronts, the map of every AIJ
// entry into a frontal matrix, the extend-add maps) is the caller's; this file
// runs the numeric phases on frontal matrices stored row-major, one after the
// other, in one device buffer.
//
// Factorisation.  Panel q's frontal matrix M (n x n) holds its P pivots first and
// its front F after them.  After the extend-add of the previous panel's Schur
// complement, the P pivot columns are eliminated by blocked Gauss-Jordan without
// pivoting, NB pivots per step:
//
//     D = M[K,K] (NB x NB),  T = D^-1 M[K,:],  C = M[:,K]
//     M[K,:] = T,   M[K,K] = D^-1,
//     M[i,K] = -C[i] D^-1,          i not in K
//     M[i,j] = M[i,j] - C[i] T[j],  i, j not in K
//
// After the P pivots M = [A^-1, A^-1 B; -C A^-1, S] with A = M[P,P], B = M[P,F],
// C = M[F,P] and S = M[F,F] - C A^-1 B the Schur complement passed on to the
// next panel.  Gauss-Jordan does about twice the work of a partial LU on these
// matrices, but every step is one parallel rank-NB update (no triangular solves,
// whose column-by-column latency dominates dense LU at these sizes), and it
// leaves exactly what the solve needs as dense blocks.  Without pivoting the
// elimination needs a nonzero pivot in every step: a pivot below tol times the
// largest entry of its NB x NB block sets an error flag and the caller
// factorises that matrix another way.
//
// Solve (two launches per panel, replayed from a CUDA graph): forward
// y_P = A^-1 b_P, b_F += (-C A^-1) b_P; backward x_P = y_P - (A^-1 B) x_F.  Sums
// run in a fixed order (warp-strided, then a fixed shuffle tree): results are
// reproducible run to run.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "vefem.h"

namespace {

constexpr int NB = 16;   // pivots per Gauss-Jordan step
constexpr int TILE = 32; // output tile of the update kernel (TILE x TILE)

// Positive doubles order like their bit patterns: atomicMin on the bits.
__device__ void atomic_min_pos(unsigned long long *addr, double v)
{
    atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

// 1/x: a single-precision seed refined by two steps of Newton's iteration for
// the reciprocal, r <- r + r (1 - x r) (quadratic convergence: ~2^-23 ->
// ~2^-46 -> rounding level).  A handful of FP64 instructions instead of a full
// IEEE division, which matters on the critical path of the pivot-block
// inversion (FP64 instructions issue at 2 lanes per clock per SM on this GPU).
// Values outside the single-precision range take the IEEE division.
__device__ __forceinline__ double recip(double x)
{
    const float xf = (float)x;
    const float rf = __frcp_rn(xf);
    if (!(fabsf(rf) < 3.0e38f) || rf == 0.0f || !(fabsf(xf) < 3.0e38f)) return 1.0 / x;
    double r = (double)rf;
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// D^-1 of the kb x kb block at M[k0][k0] (leading dimension n) by Gauss-Jordan
// without pivoting, in one warp: lane c owns column c of [D | I] (D padded to
// NB x NB with the identity), kept in shared memory column-major (padded
// stride: no bank conflicts).  The pivot loop is not unrolled (compact code:
// it runs once per launch, so a long unrolled body would mostly wait for
// instruction fetches).  The inverse lands in inv[NB][NB] (shared, row-major).
// A pivot at most tol times the largest |entry| of the block (or not finite)
// sets *err; the smallest |pivot| / largest |entry| goes to *minpiv.
__device__ void warp_invert(const double *__restrict__ M, int64_t n, int k0, int kb, double tol,
                            double (*A)[NB + 1], double (*inv)[NB], int *err,
                            unsigned long long *minpiv, bool report)
{
    const int c = threadIdx.x & 31;
    double amax = 0.0;
#pragma unroll
    for (int r = 0; r < NB; r++) {
        double v;
        if (c < NB)
            v = (r < kb && c < kb) ? M[(int64_t)(k0 + r) * n + k0 + c] : (r == c ? 1.0 : 0.0);
        else
            v = (r == c - NB) ? 1.0 : 0.0;
        A[c][r] = v;
        if (c < kb && r < kb) amax = fmax(amax, fabs(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    __syncwarp();
    bool bad = !(amax > 0.0) || !isfinite(amax);
    const double floor_ = tol * amax;
    double pmin = INFINITY;
#pragma unroll 1
    for (int p = 0; p < NB; p++) {
        double f[NB];
#pragma unroll
        for (int r = 0; r < NB; r++) f[r] = A[p][r];      // column p (broadcast reads)
        const double piv = A[p][p];
        if (p < kb) {
            const double ap = fabs(piv);
            pmin = fmin(pmin, ap);
            if (!(ap > floor_) || !isfinite(piv)) bad = true;
        }
        const double rp = A[c][p] * recip(piv);
        __syncwarp();
#pragma unroll
        for (int r = 0; r < NB; r++) A[c][r] = (r == p) ? rp : fma(-f[r], rp, A[c][r]);
        __syncwarp();
    }
    if (c >= NB) {
#pragma unroll
        for (int r = 0; r < NB; r++) inv[r][c - NB] = A[c][r];
    }
    if (report && c == 0) {
        if (bad) atomicExch(err, 1);
        const double rel = pmin / amax;
        if (rel < INFINITY && isfinite(rel)) atomic_min_pos(minpiv, rel);
    }
}

// Step part 1: D^-1 (every CTA, one warp), T = D^-1 M[K,:] for the CTA's 16
// columns (written to Tbuf and into the pivot rows of M, pivot columns left
// for part 2), and the copy C = M[:,K] of the CTA's 16 rows.
__global__ void __launch_bounds__(128) k_gj_prep(double *__restrict__ M, int n, int k0, int kb,
                                                 double *__restrict__ Tbuf, double *__restrict__ Cbuf,
                                                 double *__restrict__ invbuf, int *err,
                                                 unsigned long long *minpiv, double tol)
{
    __shared__ double sA[32][NB + 1];
    __shared__ double sInv[NB][NB];
    const int t = threadIdx.x;
    if (t < 32) warp_invert(M, n, k0, kb, tol, sA, sInv, err, minpiv, blockIdx.x == 0);
    __syncthreads();
    // the inverse for the update kernel (padded rows/columns are the identity's)
    if (blockIdx.x == 0)
        for (int u = t; u < NB * NB; u += blockDim.x) invbuf[u] = sInv[u / NB][u % NB];
    // T for columns j0..j0+15: thread = (column, pair of pivot rows)
    const int j = blockIdx.x * 16 + (t & 15);
    const int g = t >> 4;
    if (j < n && (j < k0 || j >= k0 + kb)) {
        double m[NB];
#pragma unroll
        for (int l = 0; l < NB; l++) m[l] = l < kb ? M[(int64_t)(k0 + l) * n + j] : 0.0;
#pragma unroll
        for (int kk = 0; kk < 2; kk++) {
            const int k = g * 2 + kk;
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < NB; l++) s = fma(sInv[k][l], m[l], s);
            Tbuf[(int64_t)k * n + j] = s;
            if (k < kb) M[(int64_t)(k0 + k) * n + j] = s;
        }
    }
    // C = M[i, K] for rows i0..i0+15
    for (int u = t; u < 16 * NB; u += blockDim.x) {
        const int i = blockIdx.x * 16 + u / NB, l = u % NB;
        if (i < n) Cbuf[(int64_t)i * NB + l] = l < kb ? M[(int64_t)i * n + k0 + l] : 0.0;
    }
}

// Step part 2: every entry outside the pivot rows (and the pivot block itself).
__global__ void __launch_bounds__(256) k_gj_update(double *__restrict__ M, int n, int k0, int kb,
                                                   const double *__restrict__ Tbuf,
                                                   const double *__restrict__ Cbuf,
                                                   const double *__restrict__ invbuf)
{
    __shared__ double sC[TILE][NB + 1];
    __shared__ double sT[NB][TILE];
    __shared__ double sInv[NB][NB];
    const int t = threadIdx.x;
    const int i0 = blockIdx.y * TILE, j0 = blockIdx.x * TILE;
    for (int u = t; u < TILE * NB; u += blockDim.x) {
        const int r = u / NB, l = u % NB;
        sC[r][l] = (i0 + r < n) ? Cbuf[(int64_t)(i0 + r) * NB + l] : 0.0;
        const int k = u / TILE, c = u % TILE;
        sT[k][c] = (j0 + c < n) ? Tbuf[(int64_t)k * n + j0 + c] : 0.0;
    }
    if (t < NB * NB) sInv[t / NB][t % NB] = invbuf[t];
    __syncthreads();
    const int r = t >> 3;            // tile row
    const int c0 = (t & 7) * 4;      // 4 consecutive tile columns
    const int i = i0 + r;
    if (i >= n) return;
    const bool iK = i >= k0 && i < k0 + kb;
    double ci[NB];
#pragma unroll
    for (int l = 0; l < NB; l++) ci[l] = sC[r][l];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int c = c0 + u, j = j0 + c;
        if (j >= n) continue;
        const bool jK = j >= k0 && j < k0 + kb;
        double *dst = M + (int64_t)i * n + j;
        if (iK) {
            if (jK) *dst = sInv[i - k0][j - k0];
            continue;                // the rest of the pivot rows: part 1
        }
        if (jK) {
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < NB; l++) s = fma(ci[l], sInv[l][j - k0], s);
            *dst = -s;
        } else {
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < NB; l++) s = fma(ci[l], sT[l][c], s);
            *dst = *dst - s;
        }
    }
}

// M_q[e[a], e[b]] += S_prev[a, b], S_prev = M_prev[p_prev:, p_prev:]
__global__ void k_extend_add(double *__restrict__ Mq, int nq, const double *__restrict__ Mp, int np,
                             int pp, const int32_t *__restrict__ e, int f)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)f * f) return;
    const int a = (int)(t / f), b = (int)(t - (int64_t)a * f);
    Mq[(int64_t)e[a] * nq + e[b]] += Mp[(int64_t)(pp + a) * np + pp + b];
}

__device__ double warp_sum(double s)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// forward: row r of M[:, :p] against b_P; r < p -> y, r >= p -> b_F +=
__global__ void k_solve_fwd(const double *__restrict__ M, int n, int p, const int64_t *__restrict__ idx,
                            double *__restrict__ b, double *__restrict__ y)
{
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    const double *row = M + (int64_t)r * n;
    double s = 0.0;
    for (int c = lane; c < p; c += 32) s = fma(row[c], b[idx[c]], s);
    s = warp_sum(s);
    if (lane == 0) {
        if (r < p)
            y[idx[r]] = s;
        else
            b[idx[r]] += s;
    }
}

// backward: x_P = y_P - M[:p, p:] x_F
__global__ void k_solve_bwd(const double *__restrict__ M, int n, int p, const int64_t *__restrict__ idx,
                            const double *__restrict__ y, double *__restrict__ x)
{
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= p) return;
    const double *row = M + (int64_t)r * n + p;
    const int f = n - p;
    double s = 0.0;
    for (int c = lane; c < f; c += 32) s = fma(row[c], x[idx[p + c]], s);
    s = warp_sum(s);
    if (lane == 0) x[idx[r]] = y[idx[r]] - s;
}

}  // namespace

struct vefem_frontal {
    int device = 0;
    int npan = 0;
    int64_t N = 0;
    int nmax = 0;
    std::vector<int64_t> off, ext_off, idx_off;
    std::vector<int> n, p;
    const int32_t *ext = nullptr;   // caller's device arrays
    const int64_t *idx = nullptr;
    double *Tbuf = nullptr, *Cbuf = nullptr, *inv = nullptr;
    int *err = nullptr;
    unsigned long long *minpiv = nullptr;
    unsigned long long h_minpiv = 0;   // staging of the initial value (outlives the async copy)
    // solve: work vectors and the CUDA graph of the two sweeps (captured per buf)
    double *wb = nullptr, *wy = nullptr, *wx = nullptr;
    cudaStream_t cs = nullptr;
    cudaGraphExec_t graph = nullptr;
    const double *graph_buf = nullptr;
    std::string msg;
};

namespace {

int ffail(vefem_frontal *f, int code, const std::string &m)
{
    if (f) f->msg = m;
    return code;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int d)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(d);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

#define FCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess)                                                           \
            return ffail(f, VEFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

extern "C" int vefem_frontal_create(int device, int npan, const int64_t *off, const int32_t *n,
                                    const int32_t *p, const int32_t *ext, const int64_t *ext_off,
                                    const int64_t *idx, const int64_t *idx_off, int64_t N,
                                    vefem_frontal **out)
{
    if (!out || npan <= 0 || !off || !n || !p || !ext_off || !idx || !idx_off || N <= 0 ||
        (npan > 1 && !ext))
        return VEFEM_ERR_ARG;
    *out = nullptr;
    vefem_frontal *f = new vefem_frontal();
    f->device = device;
    f->npan = npan;
    f->N = N;
    f->off.assign(off, off + npan + 1);
    f->ext_off.assign(ext_off, ext_off + npan);
    f->idx_off.assign(idx_off, idx_off + npan + 1);
    f->n.assign(n, n + npan);
    f->p.assign(p, p + npan);
    f->ext = ext;
    f->idx = idx;
    int64_t tot = 0;
    for (int q = 0; q < npan; q++) {
        if (n[q] <= 0 || p[q] < 0 || p[q] > n[q] || f->off[q + 1] - f->off[q] != (int64_t)n[q] * n[q] ||
            f->idx_off[q + 1] - f->idx_off[q] != n[q]) {
            delete f;
            return VEFEM_ERR_ARG;
        }
        if (q + 1 < npan && n[q] - p[q] > n[q + 1]) {   // the front must fit in the next panel
            delete f;
            return VEFEM_ERR_ARG;
        }
        tot += p[q];
        f->nmax = std::max(f->nmax, n[q]);
    }
    if (tot != N) {            // every unknown is a pivot exactly once
        delete f;
        return VEFEM_ERR_ARG;
    }
    DeviceGuard g(device);
    if (cudaMalloc(&f->wb, (size_t)N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->wy, (size_t)N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->wx, (size_t)N * sizeof(double)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&f->cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&f->Tbuf, (size_t)NB * f->nmax * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->Cbuf, (size_t)NB * f->nmax * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->inv, NB * NB * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->err, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&f->minpiv, sizeof(unsigned long long)) != cudaSuccess) {
        vefem_frontal_destroy(f);
        return VEFEM_ERR_NOMEM;
    }
    *out = f;
    return VEFEM_OK;
}

extern "C" int vefem_frontal_factor(vefem_frontal *f, double *buf, void *stream, double tol,
                                    double *min_pivot)
{
    if (!f || !buf) return VEFEM_ERR_ARG;
    DeviceGuard g(f->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FCK(cudaMemsetAsync(f->err, 0, sizeof(int), s));
    const double d_one = 1.0;
    std::memcpy(&f->h_minpiv, &d_one, sizeof(d_one));
    FCK(cudaMemcpyAsync(f->minpiv, &f->h_minpiv, sizeof(f->h_minpiv), cudaMemcpyHostToDevice, s));
    for (int q = 0; q < f->npan; q++) {
        const int n = f->n[q], p = f->p[q];
        double *M = buf + f->off[q];
        if (q > 0) {
            const int np = f->n[q - 1], pp = f->p[q - 1], fr = np - pp;
            if (fr > 0) {
                const int64_t tot = (int64_t)fr * fr;
                k_extend_add<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
                    M, n, buf + f->off[q - 1], np, pp, f->ext + f->ext_off[q - 1], fr);
            }
        }
        const unsigned gp = (unsigned)((n + 15) / 16);
        const dim3 gu((unsigned)((n + TILE - 1) / TILE), (unsigned)((n + TILE - 1) / TILE));
        for (int k0 = 0; k0 < p; k0 += NB) {
            const int kb = std::min(NB, p - k0);
            k_gj_prep<<<gp, 128, 0, s>>>(M, n, k0, kb, f->Tbuf, f->Cbuf, f->inv, f->err, f->minpiv, tol);
            k_gj_update<<<gu, 256, 0, s>>>(M, n, k0, kb, f->Tbuf, f->Cbuf, f->inv);
        }
    }
    FCK(cudaGetLastError());
    int herr = 0;
    unsigned long long hmin = 0;
    FCK(cudaMemcpyAsync(&herr, f->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    FCK(cudaMemcpyAsync(&hmin, f->minpiv, sizeof(hmin), cudaMemcpyDeviceToHost, s));
    FCK(cudaStreamSynchronize(s));
    if (min_pivot) std::memcpy(min_pivot, &hmin, sizeof(double));
    if (herr) return ffail(f, VEFEM_ERR_SINGULAR, "a pivot below the tolerance (unpivoted elimination)");
    return VEFEM_OK;
}

namespace {

// the two sweeps of a solve, on stream s, with the handle's work vectors
void launch_sweeps(vefem_frontal *f, const double *buf, cudaStream_t s)
{
    for (int q = 0; q < f->npan; q++) {
        const int n = f->n[q];
        if (f->p[q] == 0) continue;
        k_solve_fwd<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(buf + f->off[q], n, f->p[q],
                                                           f->idx + f->idx_off[q], f->wb, f->wy);
    }
    for (int q = f->npan - 1; q >= 0; q--) {
        const int p = f->p[q];
        if (p == 0) continue;
        k_solve_bwd<<<(unsigned)((p + 7) / 8), 256, 0, s>>>(buf + f->off[q], f->n[q], p,
                                                           f->idx + f->idx_off[q], f->wy, f->wx);
    }
}

}  // namespace

extern "C" int vefem_frontal_solve(vefem_frontal *f, const double *buf, const double *b, double *x,
                                   void *stream)
{
    if (!f || !buf || !b || !x) return VEFEM_ERR_ARG;
    DeviceGuard g(f->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!f->graph || f->graph_buf != buf) {
        // capture the 2 x npan launches once per factor buffer: a replay costs a
        // fraction of their launch overhead
        if (f->graph) {
            cudaGraphExecDestroy(f->graph);
            f->graph = nullptr;
        }
        FCK(cudaStreamBeginCapture(f->cs, cudaStreamCaptureModeThreadLocal));
        launch_sweeps(f, buf, f->cs);
        cudaGraph_t gr = nullptr;
        const cudaError_t le = cudaGetLastError();
        FCK(cudaStreamEndCapture(f->cs, &gr));
        if (le != cudaSuccess) {
            cudaGraphDestroy(gr);
            return ffail(f, VEFEM_ERR_CUDA, std::string("solve capture: ") + cudaGetErrorString(le));
        }
        const cudaError_t ie = cudaGraphInstantiate(&f->graph, gr, 0);
        cudaGraphDestroy(gr);
        if (ie != cudaSuccess) {
            f->graph = nullptr;
            return ffail(f, VEFEM_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
        }
        f->graph_buf = buf;
    }
    FCK(cudaMemcpyAsync(f->wb, b, (size_t)f->N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    FCK(cudaGraphLaunch(f->graph, s));
    FCK(cudaMemcpyAsync(x, f->wx, (size_t)f->N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return VEFEM_OK;
}

extern "C" void vefem_frontal_destroy(vefem_frontal *f)
{
    if (!f) return;
    {
        DeviceGuard g(f->device);
        if (f->graph) cudaGraphExecDestroy(f->graph);
        if (f->cs) cudaStreamDestroy(f->cs);
        cudaFree(f->wb);
        cudaFree(f->wy);
        cudaFree(f->wx);
        cudaFree(f->Tbuf);
        cudaFree(f->Cbuf);
        cudaFree(f->inv);
        cudaFree(f->err);
        cudaFree(f->minpiv);
    }
    delete f;
}

extern "C" const char *vefem_frontal_last_error(const vefem_frontal *f)
{
    return f ? f->msg.c_str() : "null frontal handle";
}
