// Exact (linearised) element Jacobian by forward-mode differentiation of the
// Gauss-point physics, in FP32 (the inexact-Newton "precision form") or FP64.
//
// At a Gauss point the weak-form term of test node i and equation e is linear
// in the test function: TERM(i,e) = sum_k c_ek(q) psi_k(i), psi = (phi, dphi/dx,
// dphi/dy), where the coefficients c (6 equations x 3) depend on the 20
// interpolated quantities q (u, v: value, x/y gradient, Laplacian; p and the
// three stress components: value, x/y gradient) and on Wi (through the
// arclength unknown).  Each unknown x(j,f) enters q linearly through chi(j) =
// (phi_j, dphi_j/dx, dphi_j/dy, Laplacian phi_j).  Hence
//     dR(i,e)/dx(j,f) = sum_gp WET sum_k psi_k(i) sum_s (dc_ek/dq_fs) chi_s(j).
// The kernel gets dc/dq with 21 one-direction dual evaluations per Gauss
// point (the kernels' own physics source with R = Dual<T>), then contracts.
// This replaces the 56 residual evaluations of the forward difference; it is
// the derivative the FD approximates (they differ by the FD truncation error).
//
// One element at a time per CTA of 192 threads (persistent: each CTA walks a
// list of work items, each a run of consecutive elements of one mesh; a
// single mesh is the one-instance case):
//   phase 0  state and geometry, then the interpolated quantities per Gauss
//            point;
//   phase 1  thread (gp, d): D[gp][d][e*3+k] = dc_ek/dq_d;
//   phase 2a A[gp][d][i*6+e] = WET sum_k psi_k(i) D[gp][d][e*3+k];
//   phase 2b K(i,e; j,f) = sum_gp sum_s A[gp][q(f,s)][i*6+e] chi_s(j), and the
//            arclength column sum_gp A[gp][20][i*6+e];
// written to the element scratch in the block layout the scatter reads.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vefem_dual.cuh"
#include "vefem_internal.h"
#include "vefem_physics.cuh"

namespace vefem {

__constant__ double x_w[9];
__constant__ double x_bfn[9][9];
__constant__ double x_dfdc[9][9];
__constant__ double x_dfde[9][9];
__constant__ double x_d2fdc2[9][9];
__constant__ double x_d2fde2[9][9];
__constant__ double x_d2fdce[9][9];
// FP32 copies for the FP32 Jacobian (its geometry runs in FP32 on coordinates
// relative to the element's first node)
__constant__ float xf_w[9];
__constant__ float xf_dfdc[9][9];
__constant__ float xf_dfde[9][9];
__constant__ float xf_d2fdc2[9][9];
__constant__ float xf_d2fde2[9][9];
__constant__ float xf_d2fdce[9][9];

cudaError_t upload_tables_exact(const GaussTables &t, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
#define UP(sym, src)                                                                       \
    if (e == cudaSuccess)                                                                  \
        e = cudaMemcpyToSymbolAsync(sym, src, sizeof(src), 0, cudaMemcpyHostToDevice, s);
    UP(x_w, t.w)
    UP(x_bfn, t.bfn)
    UP(x_dfdc, t.dfdc)
    UP(x_dfde, t.dfde)
    UP(x_d2fdc2, t.d2fdc2)
    UP(x_d2fde2, t.d2fde2)
    UP(x_d2fdce, t.d2fdce)
#undef UP
    float w[9], a[5][9][9];
    for (int i = 0; i < 9; i++) {
        w[i] = (float)t.w[i];
        for (int j = 0; j < 9; j++) {
            a[0][i][j] = (float)t.dfdc[i][j];
            a[1][i][j] = (float)t.dfde[i][j];
            a[2][i][j] = (float)t.d2fdc2[i][j];
            a[3][i][j] = (float)t.d2fde2[i][j];
            a[4][i][j] = (float)t.d2fdce[i][j];
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_w, w, sizeof(w), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_dfdc, a[0], sizeof(a[0]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_dfde, a[1], sizeof(a[1]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_d2fdc2, a[2], sizeof(a[2]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_d2fde2, a[3], sizeof(a[3]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(xf_d2fdce, a[4], sizeof(a[4]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // the host staging arrays go out of scope
    return e;
}

constexpr int EX_THREADS = 192;
constexpr int EX_NDIR = 21;      // 20 interpolated quantities + the arclength unknown
// row stride of A: 54 entries padded to 58, which cuts the shared-memory bank
// conflicts of the contraction's reads (qdir(f, s) rows at once) by a third
constexpr int EX_AST = 58;

// direction index of quantity s (0 value, 1 d/dx, 2 d/dy, 3 Laplacian) of field f
__device__ __forceinline__ int qdir(int f, int s)
{
    return f == 0 ? s : (f == 1 ? 4 + s : 8 + 3 * (f - 2) + s);
}

template <class T>
struct TView {
    const T *p;
    __device__ __forceinline__ T operator()(int pos) const { return p[pos]; }
};

template <class T, int FORM, int SPEC>
__device__ __forceinline__ void exact_element(const ElemArgs &a, const KParams &prm,
                                              T *__restrict__ es, T *__restrict__ as, const int e)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *D = reinterpret_cast<T *>(smraw);               // [9][21][18]
    T *A = D + 9 * EX_NDIR * 18;                       // [9][21][EX_AST]
    __shared__ T s_tl[54];
    __shared__ T s_dFx[9][9], s_dFy[9][9], s_d2x[9][9], s_d2y[9][9], s_lap[9][9];
    __shared__ T s_H2[9], s_WET[9];
    __shared__ T s_bfn[9][9];          // basis values in T: no FP64 conversions in the loops
    __shared__ Interp<T> s_ip[9];      // interpolated quantities per Gauss point
    const int t = threadIdx.x;
    if (t >= 96 && t < 96 + 81) s_bfn[(t - 96) / 9][(t - 96) % 9] = (T)x_bfn[(t - 96) / 9][(t - 96) % 9];

    if (t < 54) {
        const int inod = t / 6, f = t - 6 * (t / 6);
        s_tl[t] = (T)a.TL[(size_t)f * a.nnodes + a.conn[inod * a.nel + e]];
    } else if (t >= 64 && t < 73) {
        const int ig = t - 64;
        // coordinates relative to node 0 (the map's derivatives see only
        // differences), then the geometry in T
        T x[9], y[9], fx[9], fy[9], sx[9], sy[9];
        const int g0 = a.conn[e];
        const double x0 = a.xy[g0], y0 = a.xy[a.nnodes + g0];
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int gn = a.conn[n * a.nel + e];
            x[n] = (T)(a.xy[gn] - x0);
            y[n] = (T)(a.xy[a.nnodes + gn] - y0);
        }
        GeoOut<T> go;
        if constexpr (sizeof(T) == 4)
            go = geometry(xf_dfdc[ig], xf_dfdc[ig], xf_dfde[ig], xf_d2fdc2[ig], xf_d2fde2[ig],
                          xf_d2fdce[ig], xf_w[ig], x, y, fx, fy, sx, sy);
        else
            go = geometry(x_dfdc[ig], x_dfdc[ig], x_dfde[ig], x_d2fdc2[ig], x_d2fde2[ig],
                          x_d2fdce[ig], x_w[ig], x, y, fx, fy, sx, sy);
#pragma unroll
        for (int n = 0; n < 9; n++) {
            s_dFx[ig][n] = fx[n];
            s_dFy[ig][n] = fy[n];
            s_d2x[ig][n] = sx[n];
            s_d2y[ig][n] = sy[n];
            s_lap[ig][n] = sx[n] + sy[n];
        }
        s_H2[ig] = go.H2;
        s_WET[ig] = go.WET;
    }
    __syncthreads();
    // phase 0b: the 20 interpolated quantities of each Gauss point, once per
    // element (the 21 direction threads of a Gauss point share them)
    if (t < 9) {
        TView<T> V{s_tl};
        s_ip[t] = interpolate(V, s_bfn[t], s_dFx[t], s_dFy[t], s_d2x[t], s_d2y[t]);
    }
    __syncthreads();

    // phase 1: dc/dq along direction d at Gauss point gp
    if (t < 9 * EX_NDIR) {
        const int gp = t / EX_NDIR, d = t - EX_NDIR * (t / EX_NDIR);
        if (d < 20 || prm.nex > 0) {
            typedef Dual<T> R;
            const Interp<T> Ip = s_ip[gp];
            Interp<R> I;
#define SEED(field, idx) I.field = R(Ip.field, d == (idx) ? (T)1 : (T)0)
            SEED(U1, 0); SEED(GU11, 1); SEED(GU21, 2); SEED(lap1, 3);
            SEED(U2, 4); SEED(GU12, 5); SEED(GU22, 6); SEED(lap2, 7);
            SEED(P, 8); SEED(dPx, 9); SEED(dPy, 10);
            SEED(S11, 11); SEED(dS11x, 12); SEED(dS11y, 13);
            SEED(S12, 14); SEED(dS12x, 15); SEED(dS12y, 16);
            SEED(S22, 17); SEED(dS22x, 18); SEED(dS22y, 19);
#undef SEED
            R WiN = R(prm.WiN);
            if (prm.nex > 0) {
                const T wi0 = (T)prm.Wi0;
                WiN = R(wi0 * (T)a.EU[prm.nex - 1], d == 20 ? wi0 : (T)0);
            }
            R dotU[9];
            const GpCoef<R> g =
                gauss_point<FORM, SPEC>(I, prm, WiN, s_H2[gp], s_dFx[gp], s_dFy[gp], dotU);
            T *dst = D + (gp * EX_NDIR + d) * 18;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                R o[6];
                const R du = k == 0 ? R(0.0) : (k == 1 ? g.U1 : g.U2);
                test_node<FORM, SPEC>(g, prm, (T)(k == 0 ? 1 : 0), (T)(k == 1 ? 1 : 0),
                                      (T)(k == 2 ? 1 : 0), du, (T)1, o);
#pragma unroll
                for (int q = 0; q < 6; q++) dst[q * 3 + k] = o[q].d;
            }
        }
    }
    __syncthreads();

    // phase 2a: test-function side
    for (int it = t; it < 9 * EX_NDIR * 9; it += EX_THREADS) {
        const int i = it % 9;
        const int gd = it / 9;               // gp*21 + d
        const int gp = gd / EX_NDIR;
        const T *dd = D + gd * 18;
        const T b0 = s_bfn[gp][i], b1 = s_dFx[gp][i], b2 = s_dFy[gp][i], w = s_WET[gp];
        T *dst = A + gd * EX_AST + i * 6;
#pragma unroll
        for (int q = 0; q < 6; q++)
            dst[q] = w * (b0 * dd[q * 3 + 0] + b1 * dd[q * 3 + 1] + b2 * dd[q * 3 + 2]);
    }
    __syncthreads();

    // phase 2b: trial-function side.  Thread = (f, i, q), the 9 outputs of
    // trial nodes j = 0..8: every A value is read once for all 9 (a thread
    // per output read it 9 times; this phase was bound by shared-memory
    // bandwidth), the trial-side factors are warp broadcasts, and each sum
    // runs in the same order (Gauss point, then quantity).  f is the slowest
    // index, so a warp's threads agree on the Laplacian term and read
    // consecutive A entries.  The results go through shared memory (D is dead
    // here) to the block layout ((i*9 + j)*36 + q*6 + f) with coalesced stores.
    T *stage = D;
    for (int w = t; w < 324; w += EX_THREADS) {
        const int f = w / 54, iq = w - 54 * (w / 54);
        const int i = iq / 6, q = iq - 6 * (iq / 6);
        const int q0 = qdir(f, 0);
        const bool lap = f < 2;
        T acc[9];
#pragma unroll
        for (int j = 0; j < 9; j++) acc[j] = 0;
        for (int gp = 0; gp < 9; gp++) {
            const T *ag = A + gp * EX_NDIR * EX_AST + iq;
            const T a0 = ag[q0 * EX_AST], a1 = ag[(q0 + 1) * EX_AST], a2 = ag[(q0 + 2) * EX_AST];
            if (lap) {
                const T a3 = ag[(q0 + 3) * EX_AST];
#pragma unroll
                for (int j = 0; j < 9; j++) {
                    T v = acc[j];
                    v += a0 * s_bfn[gp][j];
                    v += a1 * s_dFx[gp][j];
                    v += a2 * s_dFy[gp][j];
                    v += a3 * s_lap[gp][j];
                    acc[j] = v;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 9; j++) {
                    T v = acc[j];
                    v += a0 * s_bfn[gp][j];
                    v += a1 * s_dFx[gp][j];
                    v += a2 * s_dFy[gp][j];
                    acc[j] = v;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 9; j++) stage[(i * 9 + j) * 36 + q * 6 + f] = acc[j];
    }
    __syncthreads();
    T *out = es + (size_t)e * 2916;
    for (int o = t; o < 2916; o += EX_THREADS) out[o] = stage[o];
    if (prm.nex > 0 && t < 54) {
        T acc = 0;
        for (int gp = 0; gp < 9; gp++) acc += A[(gp * EX_NDIR + 20) * EX_AST + t];
        as[(size_t)e * 54 + t] = acc;
    }
}

// persistent form over the work items of many meshes; each item is a run of
// consecutive elements of one mesh (the element-batch tile of its size class)
template <class T, int FORM, int SPEC>
__global__ void __launch_bounds__(EX_THREADS, sizeof(T) == 4 ? 3 : 1)
k_exact_batched(const BatchInst *__restrict__ insts, const WorkItem *__restrict__ work, int nwork)
{
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const ElemArgs a = insts[it.inst].ea;
        const KParams prm = insts[it.inst].prm;
        T *es = static_cast<T *>(insts[it.inst].es);
        T *as = static_cast<T *>(insts[it.inst].as);
        const int e_end = min(it.e0 + it.count, a.nel);
        for (int e = it.e0; e < e_end; e++) {
            exact_element<T, FORM, SPEC>(a, prm, es, as, e);
            __syncthreads();
        }
    }
}

template <class T, int FORM, int SPEC>
static cudaError_t go_exact_batched(const BatchInst *insts, const WorkItem *work, int nwork,
                                    int grid, cudaStream_t s)
{
    const size_t smem = sizeof(T) * (9 * EX_NDIR * 18 + 9 * EX_NDIR * EX_AST);
    cudaError_t e = cudaFuncSetAttribute(k_exact_batched<T, FORM, SPEC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_exact_batched<T, FORM, SPEC><<<grid, EX_THREADS, smem, s>>>(insts, work, nwork);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_exact_batched(const BatchInst *insts, const WorkItem *work, int nwork,
                                 int form, int spec, int grid, cudaStream_t s)
{
    if (nwork <= 0) return cudaSuccess;
#define GO(F, SP)                                                                              if (form == F && spec == SP) return go_exact_batched<T, F, SP>(insts, work, nwork, grid, s);
    GO(FORM_T, 0) GO(FORM_T, SPEC_RE0) GO(FORM_T, SPEC_DF0) GO(FORM_T, SPEC_RE0 | SPEC_DF0)
    GO(FORM_SQRT, 0) GO(FORM_SQRT, SPEC_RE0) GO(FORM_SQRT, SPEC_DF0)
    GO(FORM_SQRT, SPEC_RE0 | SPEC_DF0)
#undef GO
    return cudaErrorInvalidValue;
}

template <class T, int FORM, int SPEC>
static int occ_exact()
{
    const size_t smem = sizeof(T) * (9 * EX_NDIR * 18 + 9 * EX_NDIR * EX_AST);
    if (cudaFuncSetAttribute(k_exact_batched<T, FORM, SPEC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_exact_batched<T, FORM, SPEC>, EX_THREADS,
                                                  smem);
    return n;
}

int exact_batched_ctas_per_sm(int elem_size, int form, int spec)
{
#define OC(F, SP)                                                                              if (form == F && spec == SP)                                                                   return elem_size == 4 ? occ_exact<float, F, SP>() : occ_exact<double, F, SP>();
    OC(FORM_T, 0) OC(FORM_T, SPEC_RE0) OC(FORM_T, SPEC_DF0) OC(FORM_T, SPEC_RE0 | SPEC_DF0)
    OC(FORM_SQRT, 0) OC(FORM_SQRT, SPEC_RE0) OC(FORM_SQRT, SPEC_DF0)
    OC(FORM_SQRT, SPEC_RE0 | SPEC_DF0)
#undef OC
    return 0;
}

template cudaError_t launch_exact_batched<float>(const BatchInst *, const WorkItem *, int, int,
                                                 int, int, cudaStream_t);
template cudaError_t launch_exact_batched<double>(const BatchInst *, const WorkItem *, int, int,
                                                  int, int, cudaStream_t);


// FP32 scatter of the exact Jacobian (element order, as the FP64 one)
__global__ void k_gather_jacobian32(const GatherArgs g, const float *__restrict__ es,
                                    float *__restrict__ vals)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nblocks * 36) return;
    const int blk = (int)(t / 36);
    const int r = (int)(t - (int64_t)blk * 36);
    const int jeq = r / 6, ieq = r - 6 * (r / 6);
    const int64_t slot = g.rowptr[(int64_t)g.brow[blk] * 6 + jeq] + g.boff[blk] + ieq;
    const float acc0 = g.store ? 0.0f : vals[slot];
    vals[slot] = ordered_sum(acc0, g.bcon, g.bptr[blk], g.bptr[blk + 1],
                             [&](int c) { return es[(int64_t)c * 36 + r]; });
}

__global__ void k_gather_arclength32(const GatherArgs g, const float *__restrict__ as,
                                     float *__restrict__ vals)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nnodes * 6) return;
    const int node = (int)(t / 6), jeq = (int)(t - (int64_t)node * 6);
    const int64_t slot = g.rowptr[t + 1] - 1;
    const float acc0 = g.store ? 0.0f : vals[slot];
    vals[slot] = ordered_sum(acc0, g.ncon, g.nptr[node], g.nptr[node + 1],
                             [&](int c) { return as[(int64_t)c * 6 + jeq]; });
}

cudaError_t launch_gather_jacobian32(const GatherArgs &g, const float *es, float *vals,
                                     cudaStream_t s)
{
    const int64_t n = (int64_t)g.nblocks * 36;
    if (n == 0) return cudaSuccess;
    k_gather_jacobian32<<<(unsigned)((n + 287) / 288), 288, 0, s>>>(g, es, vals);
    return cudaGetLastError();
}

cudaError_t launch_gather_arclength32(const GatherArgs &g, const float *as, float *vals,
                                      cudaStream_t s)
{
    const int64_t n = (int64_t)g.nnodes * 6;
    if (n == 0 || g.nex == 0) return cudaSuccess;
    k_gather_arclength32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, as, vals);
    return cudaGetLastError();
}

}  // namespace vefem
