// Algorithmic FP64 operation counts of the element kernels.
//
// The kernels' own physics source (vefem_physics.cuh) is instantiated on the
// host with an op-counting scalar and driven through the same sequence of
// calls the kernels make for one element, so the counts follow the code that
// runs on the GPU.  +, -, *, / and sqrt count one each (exp counts one as
// well and is reported apart); sign changes and fabs are not counted.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "vefem.h"
#include "vefem_dual.cuh"
#include "vefem_internal.h"
#include "vefem_physics.cuh"

namespace {

struct Tally {
    int64_t add = 0, mul = 0, div = 0, sqrt = 0, exp = 0;
};
Tally *g_tally = nullptr;

struct Cd {
    double v;
    Cd() : v(0.0) {}
    Cd(double x) : v(x) {}
};
inline Cd operator+(Cd a, Cd b) { g_tally->add++; return Cd(a.v + b.v); }
inline Cd operator-(Cd a, Cd b) { g_tally->add++; return Cd(a.v - b.v); }
inline Cd operator*(Cd a, Cd b) { g_tally->mul++; return Cd(a.v * b.v); }
inline Cd operator/(Cd a, Cd b) { g_tally->div++; return Cd(a.v / b.v); }
inline Cd operator+(Cd a, double b) { return a + Cd(b); }
inline Cd operator-(Cd a, double b) { return a - Cd(b); }
inline Cd operator*(Cd a, double b) { return a * Cd(b); }
inline Cd operator/(Cd a, double b) { return a / Cd(b); }
inline Cd operator+(double a, Cd b) { return Cd(a) + b; }
inline Cd operator-(double a, Cd b) { return Cd(a) - b; }
inline Cd operator*(double a, Cd b) { return Cd(a) * b; }
inline Cd operator/(double a, Cd b) { return Cd(a) / b; }
inline Cd operator-(Cd a) { return Cd(-a.v); }
inline Cd sqrt(Cd a) { g_tally->sqrt++; return Cd(::sqrt(a.v)); }
inline Cd exp(Cd a) { g_tally->exp++; return Cd(::exp(a.v)); }
inline Cd fabs(Cd a) { return Cd(::fabs(a.v)); }
// comparisons (the dual numbers' sqrt and fabs branch on signs): not counted
inline bool operator<(Cd a, Cd b) { return a.v < b.v; }
inline bool operator>(Cd a, Cd b) { return a.v > b.v; }

}  // namespace

// parameters stay plain doubles when counting: their conversions and the
// arithmetic on parameters alone are per-launch constants, not element work
namespace vefem {
template <>
struct ScalarOf<Cd> {
    typedef double type;
};
template <>
struct ScalarOf<Dual<Cd>> {
    typedef double type;
};
}  // namespace vefem

namespace {

struct ArrView {
    const Cd *p;
    Cd operator()(int pos) const { return p[pos]; }
};

// One element of the FD kernel (want_jac) or of the residual kernel, counted in
// four parts: per-element work (state staging, geometry and, for the FD
// kernel, the cached interpolants of the original state), one evaluation that
// uses the cache (base and arclength evaluations), one evaluation that
// recomputes its perturbed field, and one FD column of differences.
template <int FORM, int SPEC>
void count_element(const vefem::KParams &prm, const vefem::GaussTables &T, int want_jac,
                   Tally *once, Tally *ev_cached, Tally *ev_field, Tally *fdiff)
{
    using namespace vefem;
    Cd x[9], y[9], tl[54];
    for (int n = 0; n < 9; n++) {
        x[n] = Cd(0.5 * (n % 3) + 0.1 * n);
        y[n] = Cd(0.5 * (n / 3) - 0.05 * n);
    }
    for (int i = 0; i < 54; i++) tl[i] = Cd(0.1 + 0.01 * i);
    Cd dFx[9][9], dFy[9][9], d2x[9][9], d2y[9][9], H2[9], WET[9];
    Interp<Cd> base[9];
    ArrView V{tl};
    g_tally = once;
    if (want_jac)
        for (int i = 0; i < 54; i++) {
            Cd vp = tl[i] + prm.eps;
            Cd r = vp - prm.eps;
            (void)r;
        }
    for (int ig = 0; ig < 9; ig++) {
        auto go = geometry(T.bfn[ig], T.dfdc[ig], T.dfde[ig], T.d2fdc2[ig], T.d2fde2[ig],
                           T.d2fdce[ig], T.w[ig], x, y, dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
        H2[ig] = go.H2;
        WET[ig] = go.WET;
        if (want_jac) base[ig] = interpolate(V, T.bfn[ig], dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
    }
    Cd WiN = prm.nex > 0 ? prm.Wi0 * Cd(1.0) : Cd(prm.WiN);
    for (int pass = 0; pass < 2; pass++) {
        g_tally = pass == 0 ? ev_cached : ev_field;
        Cd res[54];
        for (int ig = 0; ig < 9; ig++) {
            Interp<Cd> I;
            if (!want_jac)
                I = interpolate(V, T.bfn[ig], dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
            else {
                I = base[ig];
                if (pass == 1) interpolate_field(V, 3, T.bfn[ig], dFx[ig], dFy[ig], d2x[ig], d2y[ig], I);
            }
            Cd dotU[9];
            // both kernels leave out the exact-zero terms of ReN = 0 / DfN = 0
            auto g = gauss_point<FORM, SPEC>(I, prm, WiN, H2[ig], dFx[ig], dFy[ig], dotU);
            for (int n = 0; n < 9; n++) {
                Cd o[6];
                test_node<FORM, SPEC>(g, prm, T.bfn[ig][n], dFx[ig][n], dFy[ig][n], dotU[n],
                                      WET[ig], o);
                for (int f = 0; f < 6; f++) res[n * 6 + f] = res[n * 6 + f] + o[f];
            }
        }
        if (pass == 0) {
            g_tally = fdiff;
            for (int i = 0; i < 54; i++) {
                Cd d = (res[i] - res[i]) / prm.eps;
                (void)d;
            }
        }
    }
    g_tally = nullptr;
}

// One element of the exact-Jacobian kernel (vefem_exact.cu): per element the
// geometry and the interpolated quantities of the 9 Gauss points (once), and
// per Gauss point and tangent direction one dual evaluation of the Gauss-point
// physics and of the three test-function term sets (dir); the contractions of
// phases 2a/2b and the arclength sums are counted by the caller.
template <int FORM, int SPEC>
void count_exact(const vefem::KParams &prm, const vefem::GaussTables &T, Tally *once, Tally *dir)
{
    using namespace vefem;
    typedef Dual<Cd> R;
    Cd x[9], y[9], tl[54];
    for (int n = 0; n < 9; n++) {
        x[n] = Cd(0.5 * (n % 3) + 0.1 * n);
        y[n] = Cd(0.5 * (n / 3) - 0.05 * n);
    }
    for (int i = 0; i < 54; i++) tl[i] = Cd(0.1 + 0.01 * i);
    Cd dFx[9][9], dFy[9][9], d2x[9][9], d2y[9][9], H2[9], WET[9];
    Interp<Cd> ip[9];
    ArrView V{tl};
    g_tally = once;
    for (int ig = 0; ig < 9; ig++) {
        auto go = geometry(T.bfn[ig], T.dfdc[ig], T.dfde[ig], T.d2fdc2[ig], T.d2fde2[ig],
                           T.d2fdce[ig], T.w[ig], x, y, dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
        H2[ig] = go.H2;
        WET[ig] = go.WET;
        ip[ig] = interpolate(V, T.bfn[ig], dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
    }
    g_tally = dir;
    const Interp<Cd> &P = ip[4];
    Interp<R> I;
    I.U1 = R(P.U1, Cd(1.0)); I.GU11 = R(P.GU11, Cd(0.0)); I.GU21 = R(P.GU21, Cd(0.0));
    I.lap1 = R(P.lap1, Cd(0.0)); I.U2 = R(P.U2, Cd(0.0)); I.GU12 = R(P.GU12, Cd(0.0));
    I.GU22 = R(P.GU22, Cd(0.0)); I.lap2 = R(P.lap2, Cd(0.0)); I.P = R(P.P, Cd(0.0));
    I.dPx = R(P.dPx, Cd(0.0)); I.dPy = R(P.dPy, Cd(0.0)); I.S11 = R(P.S11, Cd(0.0));
    I.dS11x = R(P.dS11x, Cd(0.0)); I.dS11y = R(P.dS11y, Cd(0.0)); I.S12 = R(P.S12, Cd(0.0));
    I.dS12x = R(P.dS12x, Cd(0.0)); I.dS12y = R(P.dS12y, Cd(0.0)); I.S22 = R(P.S22, Cd(0.0));
    I.dS22x = R(P.dS22x, Cd(0.0)); I.dS22y = R(P.dS22y, Cd(0.0));
    R WiN = R(prm.WiN);
    if (prm.nex > 0) WiN = R(Cd(prm.Wi0) * Cd(1.0), Cd(prm.Wi0));
    // the geometry enters the dual evaluations as plain data (the kernel's
    // shared-memory tables): an operation of a dual with it counts twice
    double gx[9], gy[9];
    for (int n = 0; n < 9; n++) {
        gx[n] = dFx[4][n].v;
        gy[n] = dFy[4][n].v;
    }
    R dotU[9];
    const GpCoef<R> g = gauss_point<FORM, SPEC>(I, prm, WiN, H2[4].v, gx, gy, dotU);
    for (int k = 0; k < 3; k++) {
        R o[6];
        const R du = k == 0 ? R(0.0) : (k == 1 ? g.U1 : g.U2);
        test_node<FORM, SPEC>(g, prm, k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0,
                              du, 1.0, o);
    }
    g_tally = nullptr;
}

template <int FORM>
void count_exact_form(const vefem::KParams &k, const vefem::GaussTables &T, Tally *a, Tally *b)
{
    const int spec = (k.ReN == 0.0 ? vefem::SPEC_RE0 : 0) | (k.DfN == 0.0 ? vefem::SPEC_DF0 : 0);
    switch (spec) {
    case 0: count_exact<FORM, 0>(k, T, a, b); break;
    case 1: count_exact<FORM, 1>(k, T, a, b); break;
    case 2: count_exact<FORM, 2>(k, T, a, b); break;
    default: count_exact<FORM, 3>(k, T, a, b); break;
    }
}

template <int FORM>
void count_form(const vefem::KParams &k, const vefem::GaussTables &T, int want_jac, Tally *a,
                Tally *b, Tally *c, Tally *d)
{
    const int spec = (k.ReN == 0.0 ? vefem::SPEC_RE0 : 0) | (k.DfN == 0.0 ? vefem::SPEC_DF0 : 0);
    switch (spec) {
    case 0: count_element<FORM, 0>(k, T, want_jac, a, b, c, d); break;
    case 1: count_element<FORM, 1>(k, T, want_jac, a, b, c, d); break;
    case 2: count_element<FORM, 2>(k, T, want_jac, a, b, c, d); break;
    default: count_element<FORM, 3>(k, T, want_jac, a, b, c, d); break;
    }
}

}  // namespace

// out[0] operations per element of the element kernel selected by flags
// (VEFEM_JAC_FD64: residual + FD Jacobian, FP64; VEFEM_JAC_EXACT32 or
// VEFEM_JAC_EXACT64: the exact-Jacobian kernel alone, in its own precision;
// else the FP64 residual only), out[1..5] the split: add/sub, mul, div, sqrt,
// exp.  A fused multiply-add counts as one mul and one add.
extern "C" int vefem_algorithmic_ops(const vefem_params *p, int flags, double *out)
{
    if (!p || !out || p->form < 0 || p->form > 1 || p->model < 0 || p->model > 6) return VEFEM_ERR_ARG;
    vefem::KParams k;
    k.model = p->model; k.form = p->form; k.nex = p->nex;
    k.ReN = p->ReN; k.WiN = p->WiN; k.BvN = p->BvN; k.VeN = p->VeN; k.DfN = p->DfN;
    k.Wi0 = p->Wi0; k.dt = p->dt; k.eps = p->fd_eps;
    vefem::GaussTables T;
    vefem::gauss_tables_host(&T);
    if ((flags & (VEFEM_JAC_EXACT32 | VEFEM_JAC_EXACT64)) && !(flags & VEFEM_JAC_FD64)) {
        Tally once, dir;
        if (p->form == 1)
            count_exact_form<1>(k, T, &once, &dir);
        else
            count_exact_form<0>(k, T, &once, &dir);
        const int64_t ndir = 9 * (20 + (p->nex > 0 ? 1 : 0));
        Tally t;
        t.add = once.add + ndir * dir.add;
        t.mul = once.mul + ndir * dir.mul;
        t.div = once.div + ndir * dir.div;
        t.sqrt = once.sqrt + ndir * dir.sqrt;
        t.exp = once.exp + ndir * dir.exp;
        // phase 2a: A = WET (b0 D0 + b1 D1 + b2 D2) per (Gauss point, direction,
        // test node, field): 3 mul + 2 add + 1 mul
        const int64_t n2a = 9 * (20 + (p->nex > 0 ? 1 : 0)) * 9 * 6;
        t.mul += 4 * n2a;
        t.add += 2 * n2a;
        // phase 2b: per (trial field f, test node i, equation q, trial node j,
        // Gauss point) 4 multiply-adds for the velocity fields (Laplacian term),
        // 3 for the others
        const int64_t n2b = 9 * 6 * 9 * 9 * (2 * 4 + 4 * 3);
        t.mul += n2b;
        t.add += n2b;
        // arclength column: sums over the 9 Gauss points
        if (p->nex > 0) t.add += 54 * 9;
        out[0] = (double)(t.add + t.mul + t.div + t.sqrt + t.exp);
        out[1] = (double)t.add;
        out[2] = (double)t.mul;
        out[3] = (double)t.div;
        out[4] = (double)t.sqrt;
        out[5] = (double)t.exp;
        return VEFEM_OK;
    }
    const int want_jac = (flags & VEFEM_JAC_FD64) ? 1 : 0;
    Tally once, evc, evf, fd;
    if (p->form == 1)
        count_form<1>(k, T, want_jac, &once, &evc, &evf, &fd);
    else
        count_form<0>(k, T, want_jac, &once, &evc, &evf, &fd);
    // FD kernel: base and arclength evaluations use the cached interpolants,
    // the 54 column evaluations recompute one field; residual kernel: one
    // evaluation with full interpolation (counted in the cached slot)
    const int64_t nc = want_jac ? 1 + p->nex : 1;
    const int64_t nf = want_jac ? 54 : 0;
    const int64_t ncol = want_jac ? 54 + p->nex : 0;
    Tally t;
    t.add = once.add + nc * evc.add + nf * evf.add + ncol * fd.add;
    t.mul = once.mul + nc * evc.mul + nf * evf.mul + ncol * fd.mul;
    t.div = once.div + nc * evc.div + nf * evf.div + ncol * fd.div;
    t.sqrt = once.sqrt + nc * evc.sqrt + nf * evf.sqrt + ncol * fd.sqrt;
    t.exp = once.exp + nc * evc.exp + nf * evf.exp + ncol * fd.exp;
    // Arclength column: eu + eps and Wi0 * eu once; residual-only: the in-order
    // Gauss-point sum is counted by the accumulation above.
    if (want_jac && p->nex) t.add += 1;
    out[0] = (double)(t.add + t.mul + t.div + t.sqrt + t.exp);
    out[1] = (double)t.add;
    out[2] = (double)t.mul;
    out[3] = (double)t.div;
    out[4] = (double)t.sqrt;
    out[5] = (double)t.exp;
    return VEFEM_OK;
}
