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
//    element in shared memory; state-independent geometry (basis2D) is
//    computed once per element and Gauss point.
//  * k_res64: residual only ('MNR'): one thread per (element, Gauss point),
//    followed by an in-order sum over the Gauss points in shared memory.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "vefem_internal.h"

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

enum { FORM_T = 0, FORM_SQRT = 1 };
enum { L_PTT = 0, M_L_PTT = 1, E_PTT = 2, M_E_PTT = 3, FENE_CR = 4, FENE_P = 5, GIESEKUS = 6 };

// ---------------------------------------------------------------------------
// Geometry of one Gauss point: basis2D (Element_Calculations_mod.F90:308-361),
// Helem of setStabilizationTerms (:718-727) and WET (Equations_mod.F90:85).
// x, y: the element's 9 node coordinates.  Outputs dFx, dFy, d2x, d2y [9].
struct GeoOut {
    double H2, WET, detJ;
};

__device__ __forceinline__ GeoOut geometry(const double *bfn_unused, const double *dfdc,
                                           const double *dfde, const double *d2c,
                                           const double *d2e, const double *d2ce, double w,
                                           const double *x, const double *y, double *dFx,
                                           double *dFy, double *d2x, double *d2y)
{
    (void)bfn_unused;
    double dxdc = 0.0, dydc = 0.0, dxde = 0.0, dyde = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        dxdc = dxdc + dfdc[n] * x[n];
        dydc = dydc + dfdc[n] * y[n];
        dxde = dxde + dfde[n] * x[n];
        dyde = dyde + dfde[n] * y[n];
    }
    GeoOut g;
    g.detJ = dxdc * dyde - dxde * dydc;
    const double dcdx = dyde / g.detJ;
    const double dedx = -dydc / g.detJ;
    const double dcdy = -dxde / g.detJ;
    const double dedy = dxdc / g.detJ;
    double hs = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const double fx = (dcdx * dfdc[n] + dedx * dfde[n]);
        const double fy = (dcdy * dfdc[n] + dedy * dfde[n]);
        dFx[n] = fx;
        dFy[n] = fy;
        d2x[n] = (dcdx * dcdx) * d2c[n] + (dedx * dedx) * d2e[n] + 2.0 * dcdx * dedx * d2ce[n];
        d2y[n] = (dcdy * dcdy) * d2c[n] + (dedy * dedy) * d2e[n] + 2.0 * dcdy * dedy * d2ce[n];
        hs = hs + fx * fx + fy * fy;
    }
    const double helem = 1.0 / sqrt(hs);
    g.H2 = helem * helem;
    g.WET = w * fabs(g.detJ);
    return g;
}

// ---------------------------------------------------------------------------
// Interpolated unknowns at a Gauss point (setFlowUnknowns, :449-533).
struct Interp {
    double U1, U2, GU11, GU21, GU12, GU22, lap1, lap2, P, dPx, dPy;
    double S11, S12, S22, dS11x, dS11y, dS12x, dS12y, dS22x, dS22y;
};

// Gauss-point coefficients the test-function loop needs.
struct GpCoef {
    double U1, U2;
    double rc1, rc2;             // ReN * Convection(i)
    double P11, P12, P22;        // P_tot (P21 == P12 bit for bit)
    double M1, M2, Cont;         // Momentum, Continuity
    double tR;                   // tlsme * ReN
    double tlsme, tlsic, ntl, tlsce, tdcs, mag;
    double C11, C12, C21, C22;   // Con_EQ
    double S11, S12, S22, den;   // SQRT form: S and S11 + S22
    double WiN, fT, omb;
    double dS11x, dS11y, dS12x, dS12y, dS22x, dS22y;
};

// interpolation from a state accessor V(pos), pos = inod*6 + ieq
template <class View>
__device__ __forceinline__ Interp interpolate(const View &V, const double *bfn, const double *dFx,
                                              const double *dFy, const double *d2x,
                                              const double *d2y)
{
    Interp I;
    double u1 = 0.0, u2 = 0.0, g11 = 0.0, g21 = 0.0, g12 = 0.0, g22 = 0.0;
    double h11 = 0.0, h21 = 0.0, h12 = 0.0, h22 = 0.0, p = 0.0, px = 0.0, py = 0.0;
    double s11 = 0.0, s12 = 0.0, s22 = 0.0, a = 0.0, b = 0.0, c = 0.0, d = 0.0, e = 0.0, f = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const double t0 = V(n * 6 + 0), t1 = V(n * 6 + 1), t2 = V(n * 6 + 2);
        const double t3 = V(n * 6 + 3), t4 = V(n * 6 + 4), t5 = V(n * 6 + 5);
        const double bf = bfn[n], fx = dFx[n], fy = dFy[n], sx = d2x[n], sy = d2y[n];
        u1 = u1 + t0 * bf;
        u2 = u2 + t1 * bf;
        g11 = g11 + t0 * fx;
        g21 = g21 + t0 * fy;
        g12 = g12 + t1 * fx;
        g22 = g22 + t1 * fy;
        h11 = h11 + t0 * sx;
        h21 = h21 + t0 * sy;
        h12 = h12 + t1 * sx;
        h22 = h22 + t1 * sy;
        p = p + t2 * bf;
        px = px + t2 * fx;
        py = py + t2 * fy;
        s11 = s11 + t3 * bf;
        s12 = s12 + t4 * bf;
        s22 = s22 + t5 * bf;
        a = a + t3 * fx;
        b = b + t3 * fy;
        c = c + t4 * fx;
        d = d + t4 * fy;
        e = e + t5 * fx;
        f = f + t5 * fy;
    }
    I.U1 = u1; I.U2 = u2;
    I.GU11 = g11; I.GU21 = g21; I.GU12 = g12; I.GU22 = g22;
    I.lap1 = h11 + h21;          // G2U(1,i) + G2U(2,i) (+ G2U(3,i) = 0), strongFormMomentum :677
    I.lap2 = h12 + h22;
    I.P = p; I.dPx = px; I.dPy = py;
    I.S11 = s11; I.S12 = s12; I.S22 = s22;
    I.dS11x = a; I.dS11y = b; I.dS12x = c; I.dS12y = d; I.dS22x = e; I.dS22y = f;
    return I;
}

// Strong form and stabilisation at a Gauss point:
// strongFormEquations (:537-573), setFlowKinematics (:605-634), the
// constitutive routines (Constitutive_Models_mod.F90, Constitutive_Models_SQRT_mod.F90),
// strongFormMomentum/Continuity (:658-697), setStabilizationTerms (:701-773).
// dotU[n] = U . grad(phi_n) is returned for reuse by the test-function loop
// (the reference computes the same product there).
template <int FORM>
__device__ __forceinline__ GpCoef gauss_point(const Interp &I, const KParams &prm, double WiN,
                                              double H2, const double *dFx, const double *dFy,
                                              double *dotU)
{
    GpCoef g;
    const double BvN = prm.BvN, ReN = prm.ReN, VeN = prm.VeN, DfN = prm.DfN;
    const double omb = 1.0 - BvN;
    g.omb = omb;
    g.WiN = WiN;
    g.U1 = I.U1;
    g.U2 = I.U2;
    // setFlowKinematics, N = 2
    const double tr = I.GU11 + I.GU22;
    const double trh = tr / 2.0;
    const double gt11 = I.GU11 - trh, gt22 = I.GU22 - trh;   // GU_tr diagonal
    const double Gd11 = gt11 + gt11, Gd22 = gt22 + gt22;     // G_dot_tr
    const double Gd12 = I.GU12 + I.GU21;
    const double S11 = I.S11, S12 = I.S12, S22 = I.S22;
    g.S11 = S11; g.S12 = S12; g.S22 = S22;
    g.dS11x = I.dS11x; g.dS11y = I.dS11y; g.dS12x = I.dS12x; g.dS12y = I.dS12y;
    g.dS22x = I.dS22x; g.dS22y = I.dS22y;

    double f1, f2, f3, fT;
    double divT1, divT2, C11, C12, C21, C22, C33 = 0.0, ddT, ddS, ddC;
    // UCD convective part U . grad S (identical in both forms)
    const double u11 = I.U1 * I.dS11x + I.U2 * I.dS11y;
    const double u12 = I.U1 * I.dS12x + I.U2 * I.dS12y;
    const double u22 = I.U1 * I.dS22x + I.U2 * I.dS22y;
    if (FORM == FORM_T) {
        // strongFormConEQ (Constitutive_Models_mod.F90:55-92): T_ve = S, dTdXi = dSdXi
        const double trT = S11 + S22;
        double MDfDt = 0.0;
        if (prm.model == FENE_CR || prm.model == FENE_P) {
            // setFENEMaterialDerivative :272-311 (steady)
            const double dfx0 = I.dS11x + I.dS22x, dfy0 = I.dS11y + I.dS22y;
            const double den = (prm.model == FENE_P) ? VeN : (VeN - 2.0);
            const double dfx = (WiN / omb) * dfx0 / den;
            const double dfy = (WiN / omb) * dfy0 / den;
            MDfDt = I.U1 * dfx + I.U2 * dfy;
        }
        switch (prm.model) {
        case L_PTT:
            fT = 1.0 + (VeN * WiN * trT) / omb;
            f1 = 1.0; f2 = fT; f3 = 0.0;
            break;
        case M_L_PTT:
            fT = 1.0 + (VeN * WiN * trT) / omb;
            f1 = fT; f2 = fT; f3 = 0.0;
            break;
        case E_PTT:
            fT = exp(VeN * WiN * trT / omb);
            f1 = 1.0; f2 = fT; f3 = 0.0;
            break;
        case M_E_PTT:
            fT = exp(VeN * WiN * trT / omb);
            f1 = fT; f2 = fT; f3 = 0.0;
            break;
        case GIESEKUS:
            fT = VeN * WiN / omb;
            f1 = 1.0; f2 = 1.0; f3 = fT;
            break;
        case FENE_CR:
            fT = 1.0 + ((WiN * trT / omb)) / (VeN - 2.0);
            f1 = fT; f2 = fT - (WiN * MDfDt / fT); f3 = 0.0;
            break;
        default:  // FENE_P
            fT = 1.0 + (WiN * trT / omb) / VeN;
            f1 = 1.0; f2 = fT - (WiN * MDfDt / fT); f3 = 0.0;
            break;
        }
        const double term_I = (prm.model == FENE_P) ? MDfDt / fT : 0.0;
        // setStressTensor :344
        g.P11 = (S11 + BvN * Gd11) - I.P;
        g.P12 = S12 + BvN * Gd12;
        g.P22 = (S22 + BvN * Gd22) - I.P;
        // setUpperConvectedDerivativeT :315-331
        const double m1_11 = gt11 * S11 + I.GU21 * S12, m1_12 = gt11 * S12 + I.GU21 * S22;
        const double m1_21 = I.GU12 * S11 + gt22 * S12, m1_22 = I.GU12 * S12 + gt22 * S22;
        const double m2_11 = S11 * gt11 + S12 * I.GU21, m2_12 = S11 * I.GU12 + S12 * gt22;
        const double m2_21 = S12 * gt11 + S22 * I.GU21, m2_22 = S12 * I.GU12 + S22 * gt22;
        const double ucd11 = (u11 - m1_11) - m2_11, ucd12 = (u12 - m1_12) - m2_12;
        const double ucd21 = (u12 - m1_21) - m2_21, ucd22 = (u22 - m1_22) - m2_22;
        const double q11 = S11 * S11 + S12 * S12, q12 = S11 * S12 + S12 * S22;
        const double q22 = S12 * S12 + S22 * S22;
        const double fo = f1 * omb;
        C11 = ((WiN * ucd11 + f3 * q11) + f2 * S11) - fo * (Gd11 + term_I);
        C12 = ((WiN * ucd12 + f3 * q12) + f2 * S12) - fo * Gd12;
        C21 = ((WiN * ucd21 + f3 * q12) + f2 * S12) - fo * Gd12;
        C22 = ((WiN * ucd22 + f3 * q22) + f2 * S22) - fo * (Gd22 + term_I);
        if (prm.model == FENE_P) C33 = -(fo * term_I);
        divT1 = I.dS11x + I.dS12y;
        divT2 = I.dS12x + I.dS22y;
        ddT = ((S11 * S11 + S12 * S12) + S12 * S12) + S22 * S22;
        ddS = ddT;
        ddC = ddT;
    } else {
        // strongFormConEQ_SQRT (Constitutive_Models_SQRT_mod.F90:120-149)
        // setCTensorSQRT :379-393
        const double Cc11 = S11 * S11 + S12 * S12, Cc12 = S11 * S12 + S12 * S22;
        const double Cc22 = S12 * S12 + S22 * S22;
        const double dC11x = (I.dS11x * S11 + I.dS12x * S12) + (S11 * I.dS11x + S12 * I.dS12x);
        const double dC12x = (I.dS11x * S12 + I.dS12x * S22) + (S11 * I.dS12x + S12 * I.dS22x);
        const double dC22x = (I.dS12x * S12 + I.dS22x * S22) + (S12 * I.dS12x + S22 * I.dS22x);
        const double dC11y = (I.dS11y * S11 + I.dS12y * S12) + (S11 * I.dS11y + S12 * I.dS12y);
        const double dC12y = (I.dS11y * S12 + I.dS12y * S22) + (S11 * I.dS12y + S12 * I.dS22y);
        const double dC22y = (I.dS12y * S12 + I.dS22y * S22) + (S12 * I.dS12y + S22 * I.dS22y);
        const double trC = Cc11 + Cc22;
        double g1 = 1.0, g2 = 1.0, dg1x = 0.0, dg1y = 0.0, dg2x = 0.0, dg2y = 0.0;
        switch (prm.model) {
        case L_PTT:
            fT = 1.0 + VeN * (trC - 2.0);
            f1 = fT; f2 = fT; f3 = 0.0;
            break;
        case M_L_PTT:
            fT = 1.0 + VeN * (trC - 2.0);
            f1 = fT; f2 = fT; f3 = 0.0;
            g1 = fT; g2 = fT;
            dg1x = VeN * (dC11x + dC22x);
            dg1y = VeN * (dC11y + dC22y);
            dg2x = dg1x; dg2y = dg1y;
            break;
        case E_PTT:
            fT = exp(VeN * (trC - 2.0));
            f1 = fT; f2 = fT; f3 = 0.0;
            break;
        case M_E_PTT:
            fT = exp(VeN * (trC - 2.0));
            f1 = fT; f2 = fT; f3 = 0.0;
            g1 = fT; g2 = fT;
            dg1x = VeN * fT * (dC11x + dC22x);
            dg1y = VeN * fT * (dC11y + dC22y);
            dg2x = dg1x; dg2y = dg1y;
            break;
        case GIESEKUS:
            fT = 1.0 - 2.0 * VeN;
            f1 = 1.0 - VeN; f2 = 1.0 - 2.0 * VeN; f3 = VeN;
            break;
        case FENE_CR:
            fT = (VeN - 2.0) / (VeN - trC);
            f1 = fT; f2 = fT; f3 = 0.0;
            g1 = fT; g2 = fT;
            dg1x = fT * (dC11x + dC22x) / (VeN - trC);
            dg1y = fT * (dC11y + dC22y) / (VeN - trC);
            dg2x = dg1x; dg2y = dg1y;
            break;
        default:  // FENE_P
            fT = (VeN - 2.0) / (VeN - trC);
            f1 = 1.0; f2 = fT; f3 = 0.0;
            g1 = 1.0; g2 = fT;
            dg2x = fT * (dC11x + dC22x) / (VeN - trC);
            dg2y = fT * (dC11y + dC22y) / (VeN - trC);
            break;
        }
        // setStressTensorSQRT :483-509
        const double rr = omb / WiN;
        const double T11 = rr * (g2 * Cc11 - g1), T12 = rr * (g2 * Cc12);
        const double T22 = rr * (g2 * Cc22 - g1), T33 = rr * (-g1);
        g.P11 = (T11 + BvN * Gd11) - I.P;
        g.P12 = T12 + BvN * Gd12;
        g.P22 = (T22 + BvN * Gd22) - I.P;
        const double dT11x = rr * ((dg2x * Cc11 + g2 * dC11x) - dg1x);
        const double dT12y = rr * (dg2y * Cc12 + g2 * dC12y);
        const double dT12x = rr * (dg2x * Cc12 + g2 * dC12x);
        const double dT22y = rr * ((dg2y * Cc22 + g2 * dC22y) - dg1y);
        divT1 = dT11x + dT12y;
        divT2 = dT12x + dT22y;
        // setUpperConvectedDerivativeSQRT :397-416 with WTensor2D :513-530
        const double den = S11 + S22;
        const double nW = (-(S11 * I.GU12) + S12 * (gt11 - gt22)) + S22 * I.GU21;
        const double W12 = nW / den;
        const double W21 = -W12;
        const double m1_11 = S11 * gt11 + S12 * I.GU21, m1_12 = S11 * I.GU12 + S12 * gt22;
        const double m1_21 = S12 * gt11 + S22 * I.GU21, m1_22 = S12 * I.GU12 + S22 * gt22;
        const double ucd11 = (u11 - m1_11) - W12 * S12, ucd12 = (u12 - m1_12) - W12 * S22;
        const double ucd21 = (u12 - m1_21) - W21 * S11, ucd22 = (u22 - m1_22) - W21 * S12;
        // setSInverse :459-479 (inverseTensor2D, Tools_mod.F90:129-146)
        const double det = S11 * S22 - S12 * S12;
        const double SI11 = S22 / det, SI12 = (-S12) / det, SI22 = S11 / det;
        const double s3_11 = S11 * Cc11 + S12 * Cc12, s3_12 = S11 * Cc12 + S12 * Cc22;
        const double s3_21 = S12 * Cc11 + S22 * Cc12, s3_22 = S12 * Cc12 + S22 * Cc22;
        C11 = WiN * ucd11 + ((f3 * s3_11 + f2 * S11) - f1 * SI11) / 2.0;
        C12 = WiN * ucd12 + ((f3 * s3_12 + f2 * S12) - f1 * SI12) / 2.0;
        C21 = WiN * ucd21 + ((f3 * s3_21 + f2 * S12) - f1 * SI12) / 2.0;
        C22 = WiN * ucd22 + ((f3 * s3_22 + f2 * S22) - f1 * SI22) / 2.0;
        ddT = (((T11 * T11 + T12 * T12) + T12 * T12) + T22 * T22) + T33 * T33;
        ddS = ((S11 * S11 + S12 * S12) + S12 * S12) + S22 * S22;
        ddC = ((Cc11 * Cc11 + Cc12 * Cc12) + Cc12 * Cc12) + Cc22 * Cc22;
        g.den = den;
    }
    g.fT = fT;
    g.C11 = C11; g.C12 = C12; g.C21 = C21; g.C22 = C22;
    // strongFormMomentum :658-683, strongFormContinuity :687-697
    const double divP1 = (-I.dPx + divT1) + BvN * I.lap1;
    const double divP2 = (-I.dPy + divT2) + BvN * I.lap2;
    const double conv1 = I.U1 * I.GU11 + I.U2 * I.GU21;
    const double conv2 = I.U1 * I.GU12 + I.U2 * I.GU22;
    g.rc1 = ReN * conv1;
    g.rc2 = ReN * conv2;
    g.M1 = g.rc1 - divP1;
    g.M2 = g.rc2 - divP2;
    g.Cont = tr;
    // setStabilizationTerms :701-773
    double tsugn = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const double du = I.U1 * dFx[n] + I.U2 * dFy[n];
        dotU[n] = du;
        tsugn = tsugn + fabs(du);
    }
    const double ddG = ((Gd11 * Gd11 + Gd12 * Gd12) + Gd12 * Gd12) + Gd22 * Gd22;
    const double r = omb / WiN;
    double Ha = sqrt(r * r + 0.5 * ddT);
    Ha = Ha / sqrt(1.0 + 0.5 * ddG);
    const double a1 = ReN / prm.dt, a2 = ReN * tsugn, a3 = BvN / H2, a4 = Ha / H2;
    double tlsme = a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4;
    tlsme = 1.0 / sqrt(tlsme);
    g.tlsme = tlsme;
    g.tlsic = H2 / tlsme;
    g.tR = tlsme * ReN;
    double tdcs = 0.5 * ddS;
    if (FORM == FORM_T) tdcs = tdcs + r * r;
    tdcs = H2 / sqrt(tdcs);
    if (DfN > 1.0e-12) tdcs = 0.0;
    g.tdcs = tdcs;
    double mag = (((C11 * C11 + C12 * C21) + C21 * C12) + C22 * C22) + C33 * C33;
    mag = sqrt(0.5 * mag);
    g.mag = mag;
    const double b1 = WiN / prm.dt, b2 = WiN * tsugn, b3 = WiN * sqrt(0.5 * ddG), b4 = f2;
    const double b5 = f3 * sqrt(0.5 * ddC), b6 = tdcs * mag / H2, b7 = DfN / H2;
    double tlsce = b1 * b1 + b2 * b2 + b3 * b3 + b4 * b4 + b5 * b5 + b6 * b6 + b7 * b7;
    tlsce = 1.0 / sqrt(tlsce);
    g.tlsce = tlsce;
    g.ntl = -tlsce;
    return g;
}

// Weak-form terms of one test node n (momentumMain(SQRT), continuityBulkMain,
// stressesBulkMain(SQRT), Residuals_mod.F90:44-157, 295-490) times WET.
template <int FORM>
__device__ __forceinline__ void test_node(const GpCoef &g, const KParams &prm, double bifn,
                                          double fx, double fy, double du, double WET,
                                          double *out)
{
    const double DfN = prm.DfN;
    // momentum
    const double lme = g.tR * du;
    const double lsme1 = lme * g.M1, lsme2 = lme * g.M2;
    const double lsic1 = (g.tlsic * fx) * g.Cont, lsic2 = (g.tlsic * fy) * g.Cont;
    double lsce1, lsce2;
    if (FORM == FORM_T) {
        // LSCEMomentumT :191-219 with doubleDotProduct (A:B^T)
        const double lx = g.ntl * fx, ly = g.ntl * fy;
        lsce1 = lx * g.C11 + ly * g.C21;
        lsce2 = lx * g.C12 + ly * g.C22;
    } else {
        // LSCEMomentumSQRT :388-433
        const double S11 = g.S11, S12 = g.S12, S22 = g.S22;
        const double m1a = S11 * fx + S12 * fy;   // (S . grad phi)_1
        const double m1b = S12 * fx + S22 * fy;   // (S . grad phi)_2
        const double wa = m1b / g.den;            // W12 for i = 1
        const double wb = -(m1a / g.den);         // W12 for i = 2
        const double k = g.tlsce;
        const double omb = g.omb, Wi = g.WiN;
        // i = 1: GU_lsce column 1 = grad phi
        double u11 = -m1a - wa * S12, u12 = -(wa * S22);
        double u21 = -m1b - (-wa) * S11, u22 = -((-wa) * S12);
        double l11 = k * u11 * omb / Wi, l12 = k * u12 * omb / Wi;
        double l21 = k * u21 * omb / Wi, l22 = k * u22 * omb / Wi;
        lsce1 = ((l11 * g.C11 + l12 * g.C21) + l21 * g.C12) + l22 * g.C22;
        // i = 2: GU_lsce column 2 = grad phi
        u11 = -(wb * S12);
        u12 = -m1a - wb * S22;
        u21 = -((-wb) * S11);
        u22 = -m1b - (-wb) * S12;
        l11 = k * u11 * omb / Wi; l12 = k * u12 * omb / Wi;
        l21 = k * u21 * omb / Wi; l22 = k * u22 * omb / Wi;
        lsce2 = ((l11 * g.C11 + l12 * g.C21) + l21 * g.C12) + l22 * g.C22;
    }
    const double pd1 = g.P11 * fx + g.P12 * fy;
    const double pd2 = g.P12 * fx + g.P22 * fy;
    const double t0 = (((g.rc1 * bifn + pd1) + lsme1) + lsic1) + lsce1;
    const double t1 = (((g.rc2 * bifn + pd2) + lsme2) + lsic2) + lsce2;
    // continuity
    const double t2 = g.Cont * bifn + g.tlsme * (fx * g.M1 + fy * g.M2);
    // stresses (j,k) = (1,1), (1,2), (2,2)
    const double gd11 = g.dS11x * fx + g.dS11y * fy;
    const double gd12 = g.dS12x * fx + g.dS12y * fy;
    const double gd22 = g.dS22x * fx + g.dS22y * fy;
    double ls11 = -fx * g.M1;
    double ls12 = -fy * g.M1 - fx * g.M2;
    double ls22 = -fy * g.M2;
    double lce;
    if (FORM == FORM_T) {
        ls11 = g.tlsme * ls11 * g.omb;
        ls12 = g.tlsme * ls12 * g.omb;
        ls22 = g.tlsme * ls22 * g.omb;
        lce = g.tlsce * (g.WiN * du);
    } else {
        ls11 = g.tlsme * ls11 * g.WiN;
        ls12 = g.tlsme * ls12 * g.WiN;
        ls22 = g.tlsme * ls22 * g.WiN;
        lce = g.tlsce * (g.WiN * du + g.fT * bifn / 2.0);
    }
    const double t3 = (((g.C11 * bifn + DfN * gd11) + ls11) + lce * g.C11) + (g.tdcs * gd11) * g.mag;
    const double t4 = (((g.C12 * bifn + DfN * gd12) + ls12) + lce * g.C12) + (g.tdcs * gd12) * g.mag;
    const double t5 = (((g.C22 * bifn + DfN * gd22) + ls22) + lce * g.C22) + (g.tdcs * gd22) * g.mag;
    out[0] = t0 * WET;
    out[1] = t1 * WET;
    out[2] = t2 * WET;
    out[3] = t3 * WET;
    out[4] = t4 * WET;
    out[5] = t5 * WET;
}

// ---------------------------------------------------------------------------
// FD kernel

constexpr int FD_EPB = 4;        // elements per CTA
constexpr int FD_NEV = 56;       // evaluations per element (base + 54 + arclength)
constexpr int FD_THREADS = FD_EPB * FD_NEV;

struct FdSmem {
    double tl[FD_EPB][3][54];    // 0: original, 1: restored (x+eps)-eps, 2: perturbed x+eps
    double dFx[FD_EPB][9][9], dFy[FD_EPB][9][9], d2x[FD_EPB][9][9], d2y[FD_EPB][9][9];
    double H2[FD_EPB][9], WET[FD_EPB][9];
    double res0[FD_EPB][54];
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

template <int FORM>
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
        GeoOut go = geometry(c_bfn[ig], c_dfdc[ig], c_dfde[ig], c_d2fdc2[ig], c_d2fde2[ig],
                             c_d2fdce[ig], c_w[ig], x, y, sm.dFx[el][ig], sm.dFy[el][ig],
                             sm.d2x[el][ig], sm.d2y[el][ig]);
        sm.H2[el][ig] = go.H2;
        sm.WET[el][ig] = go.WET;
    }
    __syncthreads();

    const bool is_ac = (k == 55);
    const bool active = live && (k < 55 || (is_ac && prm.nex > 0));
    double res[54];
#pragma unroll
    for (int i = 0; i < 54; i++) res[i] = 0.0;
    if (active) {
        FdView V;
        V.orig = sm.tl[el][0];
        V.rest = sm.tl[el][1];
        V.pert = sm.tl[el][2];
        V.kk = (k == 0) ? -1 : (is_ac ? 54 : k - 1);
        double WiN = prm.WiN;
        if (prm.nex > 0) {
            const double eu = a.EU[prm.nex - 1];
            WiN = prm.Wi0 * (is_ac ? eu + eps : eu);
        }
        for (int ig = 0; ig < 9; ig++) {
            const double *dFx = sm.dFx[el][ig], *dFy = sm.dFy[el][ig];
            Interp I = interpolate(V, c_bfn[ig], dFx, dFy, sm.d2x[el][ig], sm.d2y[el][ig]);
            double dotU[9];
            GpCoef g = gauss_point<FORM>(I, prm, WiN, sm.H2[el][ig], dFx, dFy, dotU);
            const double WET = sm.WET[el][ig];
#pragma unroll
            for (int n = 0; n < 9; n++) {
                double o[6];
                test_node<FORM>(g, prm, c_bfn[ig][n], dFx[n], dFy[n], dotU[n], WET, o);
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

constexpr int RS_EPB = 8;
constexpr int RS_THREADS = RS_EPB * 9;   // 72

struct SmemView {
    const double *p;
    __device__ __forceinline__ double operator()(int pos) const { return p[pos]; }
};

template <int FORM>
__global__ void __launch_bounds__(RS_THREADS) k_res64(const ElemArgs a, const KParams prm)
{
    __shared__ double s_tl[RS_EPB][54];
    __shared__ double s_part[RS_EPB][9][54];
    const int t = threadIdx.x;
    const int el = t / 9;
    const int ig = t - el * 9;
    const int e = blockIdx.x * RS_EPB + el;
    const bool live = (t < RS_THREADS) && e < a.nel;
    // stage element states: 54 values per element, spread over the CTA
    for (int i = t; i < RS_EPB * 54; i += blockDim.x) {
        const int ee = blockIdx.x * RS_EPB + i / 54;
        const int pos = i - (i / 54) * 54;
        if (ee < a.nel) {
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
        GeoOut go = geometry(c_bfn[ig], c_dfdc[ig], c_dfde[ig], c_d2fdc2[ig], c_d2fde2[ig],
                             c_d2fdce[ig], c_w[ig], x, y, dFx, dFy, d2x, d2y);
        double WiN = prm.WiN;
        if (prm.nex > 0) WiN = prm.Wi0 * a.EU[prm.nex - 1];
        SmemView V{s_tl[el]};
        Interp I = interpolate(V, c_bfn[ig], dFx, dFy, d2x, d2y);
        double dotU[9];
        GpCoef g = gauss_point<FORM>(I, prm, WiN, go.H2, dFx, dFy, dotU);
#pragma unroll
        for (int n = 0; n < 9; n++)
            test_node<FORM>(g, prm, c_bfn[ig][n], dFx[n], dFy[n], dotU[n], go.WET,
                            &s_part[el][ig][n * 6]);
    }
    __syncthreads();
    // in-order sum over the Gauss points (Res = Res + TERM*WET, ig = 1..9)
    for (int i = t; i < RS_EPB * 54; i += blockDim.x) {
        const int le = i / 54, pos = i - (i / 54) * 54;
        const int ee = blockIdx.x * RS_EPB + le;
        if (ee >= a.nel) continue;
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) s = s + s_part[le][q][pos];
        a.rs[(size_t)ee * 54 + pos] = s;
    }
}

cudaError_t launch_residual64(const ElemArgs &a, const KParams &p, cudaStream_t s)
{
    if (a.nel <= 0) return cudaSuccess;
    const int grid = (a.nel + RS_EPB - 1) / RS_EPB;
    if (p.form == FORM_SQRT)
        k_res64<FORM_SQRT><<<grid, RS_THREADS, 0, s>>>(a, p);
    else
        k_res64<FORM_T><<<grid, RS_THREADS, 0, s>>>(a, p);
    return cudaGetLastError();
}

cudaError_t launch_fd64(const ElemArgs &a, const KParams &p, cudaStream_t s)
{
    if (a.nel <= 0) return cudaSuccess;
    const int grid = (a.nel + FD_EPB - 1) / FD_EPB;
    if (p.form == FORM_SQRT)
        k_fd64<FORM_SQRT><<<grid, FD_THREADS, 0, s>>>(a, p);
    else
        k_fd64<FORM_T><<<grid, FD_THREADS, 0, s>>>(a, p);
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
            GeoOut go = geometry(c_ebfn[side][ig], dfdc, dfde, c_ed2c[side][ig],
                                 c_ed2e[side][ig], c_ed2ce[side][ig], 0.0, x, y, dFx, dFy, d2x,
                                 d2y);
            (void)go;
            Interp I = interpolate(V, c_ebfn[side][ig], dFx, dFy, d2x, d2y);
            double dotU[9];
            GpCoef g = gauss_point<FORM>(I, prm, WiN, go.H2, dFx, dFy, dotU);
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
