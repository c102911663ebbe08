// FP64 element assembly kernels for sm_103a: residual and the reference's
// forward-difference Jacobian, bit-compatible with the sequential algorithm.
//
// This translation unit is compiled with -fmad=false: every multiply and add
// is a separately rounded IEEE binary64 operation, evaluated in the order the
// reference Fortran writes it, so residuals match the CPU restatement bit for
// bit and the FD Jacobian (differences divided by 1e-8) does too.  The 2-D
// Cylinder_2D problem (Ndim = 2, Neq = 6) is specialised: terms that the
// reference computes with a third dimension are exact zeros there and are
// left out, which changes no value.
//
// Kernel layout (GB300: FP64 is the scarce unit, so the work is arranged to
// spend FP64 operations only on what the algorithm needs):
//  * k_fd64: one CTA = 4 elements x 56 threads; thread (element, k) evaluates
//    residual number k of storeBulk (Equations_mod.F90:264-306): k = 0 the
//    base residual, k = 1..54 the column (inod, ieq) = divmod(k-1, 6), k = 55
//    the arclength column.  The element state each evaluation sees (with the
//    (x+eps)-eps restore residue of the earlier columns) is staged once per
//    element in shared memory; state-independent geometry (basis2D) and the
//    interpolants of the unperturbed state are computed once per element and
//    Gauss point, so an evaluation recomputes only its perturbed field's
//    sums (the same sums in the same order; elements with a restore residue
//    take the full path).  Terms that are exact zeros for Re = 0 or DfN = 0
//    are left out by template specialisation.
//  * k_res64: residual only ('MNR'): one thread per (element, Gauss point),
//    followed by an in-order sum over the Gauss points in shared memory.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "vefem_internal.h"
#include "vefem_physics.cuh"

namespace vefem {

__constant__ double c_w[9];
__constant__ double c_bfn[9][9];
__constant__ double c_dfdc[9][9];
__constant__ double c_dfde[9][9];
__constant__ double c_d2fdc2[9][9];
__constant__ double c_d2fde2[9][9];
__constant__ double c_d2fdce[9][9];
__constant__ double c_ew[3];
__constant__ double c_ebfn[4][3][9];
__constant__ double c_edfdc[4][3][9];
__constant__ double c_edfde[4][3][9];
__constant__ double c_ed2c[4][3][9];
__constant__ double c_ed2e[4][3][9];
__constant__ double c_ed2ce[4][3][9];

cudaError_t upload_tables(const GaussTables &t, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
#define UP(sym, src)                                                                       \
    if (e == cudaSuccess)                                                                  \
        e = cudaMemcpyToSymbolAsync(sym, src, sizeof(src), 0, cudaMemcpyHostToDevice, s);
    UP(c_w, t.w)
    UP(c_bfn, t.bfn)
    UP(c_dfdc, t.dfdc)
    UP(c_dfde, t.dfde)
    UP(c_d2fdc2, t.d2fdc2)
    UP(c_d2fde2, t.d2fde2)
    UP(c_d2fdce, t.d2fdce)
    UP(c_ew, t.ew)
    UP(c_ebfn, t.ebfn)
    UP(c_edfdc, t.edfdc)
    UP(c_edfde, t.edfde)
    UP(c_ed2c, t.ed2c)
    UP(c_ed2e, t.ed2e)
    UP(c_ed2ce, t.ed2ce)
#undef UP
    return e;
}

// ---------------------------------------------------------------------------
// FD kernel

struct SmemView {
    const double *p;
    __device__ __forceinline__ double operator()(int pos) const { return p[pos]; }
};

constexpr int FD_EPB = 4;        // elements per CTA
constexpr int FD_NEV = 56;       // evaluations per element (base + 54 + arclength)
constexpr int FD_THREADS = FD_EPB * FD_NEV;

struct FdSmem {
    double tl[FD_EPB][3][54];    // 0: original, 1: restored (x+eps)-eps, 2: perturbed x+eps
    double dFx[FD_EPB][9][9], dFy[FD_EPB][9][9], d2x[FD_EPB][9][9], d2y[FD_EPB][9][9];
    double H2[FD_EPB][9], WET[FD_EPB][9];
    Interp<double> base[FD_EPB][9];   // interpolants of the original state per Gauss point
    double res0[FD_EPB][54];
    int residue[FD_EPB];         // 1 if some (x+eps)-eps differs from x in the element
};

// the state evaluation k sees: positions before kk are restored, kk is perturbed
struct FdView {
    const double *orig, *rest, *pert;
    int kk;
    __device__ __forceinline__ double operator()(int pos) const
    {
        const double *src = pos < kk ? rest : (pos == kk ? pert : orig);
        return src[pos];
    }
};

// the same state when no restore residue exists: original except position kk
struct FdCleanView {
    const double *orig, *pert;
    int kk;
    __device__ __forceinline__ double operator()(int pos) const
    {
        return pos == kk ? pert[pos] : orig[pos];
    }
};

template <int FORM, int SPEC>
__global__ void __launch_bounds__(FD_THREADS) k_fd64(const ElemArgs a, const KParams prm)
{
    __shared__ FdSmem sm;
    const int t = threadIdx.x;
    const int el = t / FD_NEV;
    const int k = t - el * FD_NEV;
    const int e = blockIdx.x * FD_EPB + el;
    const bool live = e < a.nel;
    const double eps = prm.eps;

    // stage the element state and geometry
    if (live && k < 54) {
        const int inod = k / 6, f = k - inod * 6;
        const int gn = a.conn[inod * a.nel + e];
        const double v = a.TL[(size_t)f * a.nnodes + gn];
        const double vp = v + eps;
        sm.tl[el][0][k] = v;
        sm.tl[el][2][k] = vp;
        sm.tl[el][1][k] = vp - eps;
    }
    if (live && k >= 54 - 9 && k < 54) {
        // nine threads per element: the nine Gauss points' geometry
        const int ig = k - 45;
        double x[9], y[9];
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int gn = a.conn[n * a.nel + e];
            x[n] = a.xy[gn];
            y[n] = a.xy[a.nnodes + gn];
        }
        auto go = geometry(c_bfn[ig], c_dfdc[ig], c_dfde[ig], c_d2fdc2[ig], c_d2fde2[ig],
                           c_d2fdce[ig], c_w[ig], x, y, sm.dFx[el][ig], sm.dFy[el][ig],
                           sm.d2x[el][ig], sm.d2y[el][ig]);
        sm.H2[el][ig] = go.H2;
        sm.WET[el][ig] = go.WET;
    }
    __syncthreads();
    if (live && k < 9) {
        // interpolants of the original state, once per element and Gauss point
        SmemView V0{sm.tl[el][0]};
        sm.base[el][k] = interpolate(V0, c_bfn[k], sm.dFx[el][k], sm.dFy[el][k], sm.d2x[el][k],
                                     sm.d2y[el][k]);
    }
    if (live && k == 9) {
        int r = 0;
        for (int i = 0; i < 54; i++)
            r |= __double_as_longlong(sm.tl[el][1][i]) != __double_as_longlong(sm.tl[el][0][i]);
        sm.residue[el] = r;
    }
    __syncthreads();

    const bool is_ac = (k == 55);
    const bool active = live && (k < 55 || (is_ac && prm.nex > 0));
    double res[54];
#pragma unroll
    for (int i = 0; i < 54; i++) res[i] = 0.0;
    if (active) {
        const int kk = (k == 0) ? -1 : (is_ac ? 54 : k - 1);
        const int fk = kk >= 0 && kk < 54 ? kk - 6 * (kk / 6) : -1;
        double WiN = prm.WiN;
        if (prm.nex > 0) {
            const double eu = a.EU[prm.nex - 1];
            WiN = prm.Wi0 * (is_ac ? eu + eps : eu);
        }
        const bool residue = sm.residue[el] != 0;
        for (int ig = 0; ig < 9; ig++) {
            const double *dFx = sm.dFx[el][ig], *dFy = sm.dFy[el][ig];
            Interp<double> I;
            if (!residue) {
                // unperturbed fields from the cache; the perturbed field recomputed
                I = sm.base[el][ig];
                if (fk >= 0) {
                    FdCleanView V{sm.tl[el][0], sm.tl[el][2], kk};
                    interpolate_field(V, fk, c_bfn[ig], dFx, dFy, sm.d2x[el][ig], sm.d2y[el][ig],
                                      I);
                }
            } else {
                FdView V;
                V.orig = sm.tl[el][0];
                V.rest = sm.tl[el][1];
                V.pert = sm.tl[el][2];
                V.kk = kk;
                I = interpolate(V, c_bfn[ig], dFx, dFy, sm.d2x[el][ig], sm.d2y[el][ig]);
            }
            double dotU[9];
            auto g = gauss_point<FORM, SPEC>(I, prm, WiN, sm.H2[el][ig], dFx, dFy, dotU);
            const double WET = sm.WET[el][ig];
#pragma unroll
            for (int n = 0; n < 9; n++) {
                double o[6];
                test_node<FORM, SPEC>(g, prm, c_bfn[ig][n], dFx[n], dFy[n], dotU[n], WET, o);
#pragma unroll
                for (int f = 0; f < 6; f++) res[n * 6 + f] = res[n * 6 + f] + o[f];
            }
        }
    }
    if (active && k == 0) {
#pragma unroll
        for (int i = 0; i < 54; i++) {
            sm.res0[el][i] = res[i];
            a.rs[(size_t)e * 54 + i] = res[i];
        }
    }
    __syncthreads();
    if (!active || k == 0) return;
    if (is_ac) {
#pragma unroll
        for (int i = 0; i < 54; i++) a.as[(size_t)e * 54 + i] = (res[i] - sm.res0[el][i]) / eps;
        return;
    }
    // column (inod, ieq) of TEMP_A_f; row (jnod, jeq)
    const int inod = (k - 1) / 6, ieq = (k - 1) - 6 * ((k - 1) / 6);
    double *dst = a.es + (size_t)e * 2916 + inod * 36 + ieq;
#pragma unroll
    for (int jnod = 0; jnod < 9; jnod++)
#pragma unroll
        for (int jeq = 0; jeq < 6; jeq++)
            dst[jnod * 324 + jeq * 6] = (res[jnod * 6 + jeq] - sm.res0[el][jnod * 6 + jeq]) / eps;
}

// ---------------------------------------------------------------------------
// Residual-only kernel: thread = (element, Gauss point)

// residual kernel: one thread per (element, Gauss point), RES_EPB elements per
// CTA (vefem_internal.h)
constexpr int RS_EPB = RES_EPB;
constexpr int RS_THREADS = RS_EPB * 9;
// 3 CTAs per SM requested: the compiler then keeps the SQRT form at 168
// registers (a few spilled values) instead of 252, and 4 CTAs fit per SM;
// measured 2.58 ms instead of 2.61 ms per 40,000 elements (the kernel is
// bound by the FP64 pipe, not by latency)
constexpr int RS_MIN_CTAS = 3;

// elements [e0, e0 + count) of one mesh, count <= RS_EPB; SPEC leaves out the
// exact-zero terms of ReN = 0 / DfN = 0 as the FD kernel does (same values)
template <int FORM, int SPEC>
__device__ __forceinline__ void res64_block(const ElemArgs &a, const KParams &prm, int e0,
                                            int count)
{
    __shared__ double s_tl[RS_EPB][54];
    __shared__ double s_part[RS_EPB][9][54];
    const int t = threadIdx.x;
    const int el = t / 9;
    const int ig = t - el * 9;
    const int e = e0 + el;
    const int e_end = min(e0 + count, a.nel);
    const bool live = (t < RS_THREADS) && e < e_end;
    // stage element states: 54 values per element, spread over the CTA
    for (int i = t; i < RS_EPB * 54; i += blockDim.x) {
        const int ee = e0 + i / 54;
        const int pos = i - (i / 54) * 54;
        if (ee < e_end) {
            const int inod = pos / 6, f = pos - 6 * (pos / 6);
            s_tl[i / 54][pos] = a.TL[(size_t)f * a.nnodes + a.conn[inod * a.nel + ee]];
        }
    }
    __syncthreads();
    if (live) {
        double x[9], y[9], dFx[9], dFy[9], d2x[9], d2y[9];
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int gn = a.conn[n * a.nel + e];
            x[n] = a.xy[gn];
            y[n] = a.xy[a.nnodes + gn];
        }
        auto go = geometry(c_bfn[ig], c_dfdc[ig], c_dfde[ig], c_d2fdc2[ig], c_d2fde2[ig],
                             c_d2fdce[ig], c_w[ig], x, y, dFx, dFy, d2x, d2y);
        double WiN = prm.WiN;
        if (prm.nex > 0) WiN = prm.Wi0 * a.EU[prm.nex - 1];
        SmemView V{s_tl[el]};
        auto I = interpolate(V, c_bfn[ig], dFx, dFy, d2x, d2y);
        double dotU[9];
        auto g = gauss_point<FORM, SPEC>(I, prm, WiN, go.H2, dFx, dFy, dotU);
#pragma unroll
        for (int n = 0; n < 9; n++)
            test_node<FORM, SPEC>(g, prm, c_bfn[ig][n], dFx[n], dFy[n], dotU[n], go.WET,
                                  &s_part[el][ig][n * 6]);
    }
    __syncthreads();
    // in-order sum over the Gauss points (Res = Res + TERM*WET, ig = 1..9)
    for (int i = t; i < RS_EPB * 54; i += blockDim.x) {
        const int le = i / 54, pos = i - (i / 54) * 54;
        const int ee = e0 + le;
        if (ee >= e_end) continue;
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) s = s + s_part[le][q][pos];
        a.rs[(size_t)ee * 54 + pos] = s;
    }
}

template <int FORM, int SPEC>
__global__ void __launch_bounds__(RS_THREADS, RS_MIN_CTAS) k_res64(const ElemArgs a, const KParams prm)
{
    res64_block<FORM, SPEC>(a, prm, blockIdx.x * RS_EPB, RS_EPB);
}

// persistent form over the work items of many meshes
template <int FORM, int SPEC>
__global__ void __launch_bounds__(RS_THREADS, RS_MIN_CTAS)
k_res64_batched(const BatchInst *__restrict__ insts, const WorkItem *__restrict__ work, int nwork)
{
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const ElemArgs a = insts[it.inst].ea;
        const KParams prm = insts[it.inst].prm;
        res64_block<FORM, SPEC>(a, prm, it.e0, it.count);
        __syncthreads();
    }
}

// the kernel's specialisation for the parameters: (form, which of ReN, DfN are zero)
#define RES_DISPATCH(form, spec, LAUNCH)                                                        \
    do {                                                                                        \
        if ((form) == FORM_SQRT) {                                                              \
            switch (spec) {                                                                     \
            case 0: LAUNCH(FORM_SQRT, 0); break;                                                \
            case SPEC_RE0: LAUNCH(FORM_SQRT, SPEC_RE0); break;                                  \
            case SPEC_DF0: LAUNCH(FORM_SQRT, SPEC_DF0); break;                                  \
            default: LAUNCH(FORM_SQRT, SPEC_RE0 | SPEC_DF0); break;                             \
            }                                                                                   \
        } else {                                                                                \
            switch (spec) {                                                                     \
            case 0: LAUNCH(FORM_T, 0); break;                                                   \
            case SPEC_RE0: LAUNCH(FORM_T, SPEC_RE0); break;                                     \
            case SPEC_DF0: LAUNCH(FORM_T, SPEC_DF0); break;                                     \
            default: LAUNCH(FORM_T, SPEC_RE0 | SPEC_DF0); break;                                \
            }                                                                                   \
        }                                                                                       \
    } while (0)

static int spec_of(const KParams &p)
{
    return (p.ReN == 0.0 ? SPEC_RE0 : 0) | (p.DfN == 0.0 ? SPEC_DF0 : 0);
}

cudaError_t launch_residual64(const ElemArgs &a, const KParams &p, cudaStream_t s)
{
    if (a.nel <= 0) return cudaSuccess;
    const int grid = (a.nel + RS_EPB - 1) / RS_EPB;
#define GO(F, SP) k_res64<F, SP><<<grid, RS_THREADS, 0, s>>>(a, p)
    RES_DISPATCH(p.form, spec_of(p), GO);
#undef GO
    return cudaGetLastError();
}

cudaError_t launch_residual64_batched(const BatchInst *insts, const WorkItem *work, int nwork,
                                      int form, int spec, int grid, cudaStream_t s)
{
    if (nwork <= 0) return cudaSuccess;
#define GO(F, SP) k_res64_batched<F, SP><<<grid, RS_THREADS, 0, s>>>(insts, work, nwork)
    RES_DISPATCH(form, spec, GO);
#undef GO
    return cudaGetLastError();
}

int residual_batched_ctas_per_sm(int form, int spec)
{
    int n = 0;
#define GO(F, SP) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_res64_batched<F, SP>, RS_THREADS, 0)
    RES_DISPATCH(form, spec, GO);
#undef GO
    return n;
}

template <int FORM>
static void launch_fd64_form(const ElemArgs &a, const KParams &p, int grid, cudaStream_t s)
{
    const int spec = (p.ReN == 0.0 ? SPEC_RE0 : 0) | (p.DfN == 0.0 ? SPEC_DF0 : 0);
    switch (spec) {
    case 0: k_fd64<FORM, 0><<<grid, FD_THREADS, 0, s>>>(a, p); break;
    case SPEC_RE0: k_fd64<FORM, SPEC_RE0><<<grid, FD_THREADS, 0, s>>>(a, p); break;
    case SPEC_DF0: k_fd64<FORM, SPEC_DF0><<<grid, FD_THREADS, 0, s>>>(a, p); break;
    default: k_fd64<FORM, SPEC_RE0 | SPEC_DF0><<<grid, FD_THREADS, 0, s>>>(a, p); break;
    }
}

cudaError_t launch_fd64(const ElemArgs &a, const KParams &p, cudaStream_t s)
{
    if (a.nel <= 0) return cudaSuccess;
    const int grid = (a.nel + FD_EPB - 1) / FD_EPB;
    if (p.form == FORM_SQRT)
        launch_fd64_form<FORM_SQRT>(a, p, grid, s);
    else
        launch_fd64_form<FORM_T>(a, p, grid, s);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Outlet open-BC edges (residualEdge / openBC / storeEdge, Equations_mod.F90:
// 387-554, Residuals_mod.F90:599-624, Element_Calculations_mod.F90:852-924).
// One CTA per edge, 56 threads = the 56 FD evaluations.

template <int FORM>
__global__ void __launch_bounds__(64) k_edge64(const EdgeArgs a, const KParams prm, int want_jac)
{
    __shared__ double s_tl[3][54];
    __shared__ double s_res0[54];
    const int k = threadIdx.x;
    const int ed = blockIdx.x;
    const int e = a.edge_elem[ed];
    const int side = a.edge_id[ed] - 1;
    const double eps = prm.eps;
    if (k < 54) {
        const int inod = k / 6, f = k - 6 * (k / 6);
        const double v = a.TL[(size_t)f * a.nnodes + a.conn[inod * a.nel + e]];
        const double vp = v + eps;
        s_tl[0][k] = v;
        s_tl[2][k] = vp;
        s_tl[1][k] = vp - eps;
    }
    __syncthreads();
    const bool is_ac = (k == 55);
    const bool active = (k == 0) || (want_jac && (k < 55 || (is_ac && prm.nex > 0)));
    double res[54];
#pragma unroll
    for (int i = 0; i < 54; i++) res[i] = 0.0;
    if (active) {
        FdView V;
        V.orig = s_tl[0];
        V.rest = s_tl[1];
        V.pert = s_tl[2];
        V.kk = (k == 0) ? -1 : (is_ac ? 54 : k - 1);
        double WiN = prm.WiN;
        if (prm.nex > 0) {
            const double eu = a.EU[prm.nex - 1];
            WiN = prm.Wi0 * (is_ac ? eu + eps : eu);
        }
        double x[9], y[9];
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int gn = a.conn[n * a.nel + e];
            x[n] = a.xy[gn];
            y[n] = a.xy[a.nnodes + gn];
        }
        for (int ig = 0; ig < 3; ig++) {
            double dFx[9], dFy[9], d2x[9], d2y[9];
            const double *dfdc = c_edfdc[side][ig], *dfde = c_edfde[side][ig];
            auto go = geometry(c_ebfn[side][ig], dfdc, dfde, c_ed2c[side][ig],
                                 c_ed2e[side][ig], c_ed2ce[side][ig], 0.0, x, y, dFx, dFy, d2x,
                                 d2y);
            (void)go;
            auto I = interpolate(V, c_ebfn[side][ig], dFx, dFy, d2x, d2y);
            double dotU[9];
            auto g = gauss_point<FORM>(I, prm, WiN, go.H2, dFx, dFy, dotU);
            // setEdgeQuantities: normal from the tangent of the edge
            double dxdc = 0.0, dydc = 0.0, dxde = 0.0, dyde = 0.0;
#pragma unroll
            for (int n = 0; n < 9; n++) {
                dxdc = dxdc + dfdc[n] * x[n];
                dydc = dydc + dfdc[n] * y[n];
                dxde = dxde + dfde[n] * x[n];
                dyde = dyde + dfde[n] * y[n];
            }
            double n1, n2;
            switch (side) {
            case 0: n1 = dydc; n2 = -dxdc; break;
            case 1: n1 = dyde; n2 = -dxde; break;
            case 2: n1 = -dydc; n2 = dxdc; break;
            default: n1 = -dyde; n2 = dxde; break;
            }
            const double dL = sqrt(n1 * n1 + n2 * n2);
            n1 = n1 / dL;
            n2 = n2 / dL;
            const double WET = c_ew[ig] * dL;
            // openBC: TERM(i) = -(n . (P_tot(:,i) + P I(:,i))) * bifn
            const double c1a = g.P11 + I.P, c1b = g.P12;          // column 1
            const double c2a = g.P12, c2b = g.P22 + I.P;          // column 2
            const double q1 = n1 * c1a + n2 * c1b;
            const double q2 = n1 * c2a + n2 * c2b;
#pragma unroll
            for (int n = 0; n < 9; n++) {
                const double bf = c_ebfn[side][ig][n];
                res[n * 6 + 0] = res[n * 6 + 0] + (-q1 * bf) * WET;
                res[n * 6 + 1] = res[n * 6 + 1] + (-q2 * bf) * WET;
                res[n * 6 + 2] = res[n * 6 + 2] + 0.0 * WET;
                res[n * 6 + 3] = res[n * 6 + 3] + 0.0 * WET;
                res[n * 6 + 4] = res[n * 6 + 4] + 0.0 * WET;
                res[n * 6 + 5] = res[n * 6 + 5] + 0.0 * WET;
            }
        }
    }
    if (k == 0) {
#pragma unroll
        for (int i = 0; i < 54; i++) {
            s_res0[i] = res[i];
            a.rs[(size_t)ed * 54 + i] = res[i];
        }
    }
    __syncthreads();
    if (!active || k == 0) return;
    if (is_ac) {
#pragma unroll
        for (int i = 0; i < 54; i++) a.as[(size_t)ed * 54 + i] = (res[i] - s_res0[i]) / eps;
        return;
    }
    const int inod = (k - 1) / 6, ieq = (k - 1) - 6 * ((k - 1) / 6);
    double *dst = a.es + (size_t)ed * 2916 + inod * 36 + ieq;
#pragma unroll
    for (int jnod = 0; jnod < 9; jnod++)
#pragma unroll
        for (int jeq = 0; jeq < 6; jeq++)
            dst[jnod * 324 + jeq * 6] = (res[jnod * 6 + jeq] - s_res0[jnod * 6 + jeq]) / eps;
}

cudaError_t launch_edge64(const EdgeArgs &a, const KParams &p, int want_jac, cudaStream_t s)
{
    if (a.nedge <= 0) return cudaSuccess;
    if (p.form == FORM_SQRT)
        k_edge64<FORM_SQRT><<<a.nedge, 64, 0, s>>>(a, p, want_jac);
    else
        k_edge64<FORM_T><<<a.nedge, 64, 0, s>>>(a, p, want_jac);
    return cudaGetLastError();
}

}  // namespace vefem
