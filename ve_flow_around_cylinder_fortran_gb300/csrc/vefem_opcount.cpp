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

struct ArrView {
    const Cd *p;
    Cd operator()(int pos) const { return p[pos]; }
};

template <int FORM>
void count_element(const vefem::KParams &prm, const vefem::GaussTables &T, int want_jac,
                   Tally *geo, Tally *evals, Tally *fdiff)
{
    using namespace vefem;
    Cd x[9], y[9], tl[54];
    for (int n = 0; n < 9; n++) {
        x[n] = Cd(0.5 * (n % 3) + 0.1 * n);
        y[n] = Cd(0.5 * (n / 3) - 0.05 * n);
    }
    for (int i = 0; i < 54; i++) tl[i] = Cd(0.1 + 0.01 * i);
    Cd dFx[9][9], dFy[9][9], d2x[9][9], d2y[9][9], H2[9], WET[9];
    // per element: state staging (x + eps, (x + eps) - eps) and geometry
    g_tally = geo;
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
    }
    // one residual evaluation (all evaluations of an element cost the same)
    g_tally = evals;
    Cd WiN = prm.nex > 0 ? prm.Wi0 * Cd(1.0) : Cd(prm.WiN);
    Cd res[54];
    ArrView V{tl};
    for (int ig = 0; ig < 9; ig++) {
        auto I = interpolate(V, T.bfn[ig], dFx[ig], dFy[ig], d2x[ig], d2y[ig]);
        Cd dotU[9];
        auto g = gauss_point<FORM>(I, prm, WiN, H2[ig], dFx[ig], dFy[ig], dotU);
        for (int n = 0; n < 9; n++) {
            Cd o[6];
            test_node<FORM>(g, prm, T.bfn[ig][n], dFx[ig][n], dFy[ig][n], dotU[n], WET[ig], o);
            for (int f = 0; f < 6; f++) res[n * 6 + f] = res[n * 6 + f] + o[f];
        }
    }
    // one FD column: 54 differences divided by eps
    g_tally = fdiff;
    for (int i = 0; i < 54; i++) {
        Cd d = (res[i] - res[i]) / prm.eps;
        (void)d;
    }
    g_tally = nullptr;
}

}  // namespace

// out[0] FP64 operations per element of the element kernel selected by flags
// (VEFEM_JAC_FD64: residual + FD Jacobian; else residual only), out[1..5] the
// split: add/sub, mul, div, sqrt, exp.
extern "C" int vefem_algorithmic_ops(const vefem_params *p, int flags, double *out)
{
    if (!p || !out || p->form < 0 || p->form > 1 || p->model < 0 || p->model > 6) return VEFEM_ERR_ARG;
    vefem::KParams k;
    k.model = p->model; k.form = p->form; k.nex = p->nex;
    k.ReN = p->ReN; k.WiN = p->WiN; k.BvN = p->BvN; k.VeN = p->VeN; k.DfN = p->DfN;
    k.Wi0 = p->Wi0; k.dt = p->dt; k.eps = p->fd_eps;
    vefem::GaussTables T;
    vefem::gauss_tables_host(&T);
    const int want_jac = (flags & VEFEM_JAC_FD64) ? 1 : 0;
    Tally geo, ev, fd;
    if (p->form == 1)
        count_element<1>(k, T, want_jac, &geo, &ev, &fd);
    else
        count_element<0>(k, T, want_jac, &geo, &ev, &fd);
    // evaluations per element: base (+ 54 columns + nex arclength columns)
    const int64_t nev = want_jac ? 1 + 54 + p->nex : 1;
    const int64_t ncol = want_jac ? 54 + p->nex : 0;
    Tally t;
    t.add = geo.add + nev * ev.add + ncol * fd.add;
    t.mul = geo.mul + nev * ev.mul + ncol * fd.mul;
    t.div = geo.div + nev * ev.div + ncol * fd.div;
    t.sqrt = geo.sqrt + nev * ev.sqrt + ncol * fd.sqrt;
    t.exp = geo.exp + nev * ev.exp + ncol * fd.exp;
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
