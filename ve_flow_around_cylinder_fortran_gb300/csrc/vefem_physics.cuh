// Element physics of the 2-D Cylinder_2D problem (Ndim = 2, Neq = 6): the
// Gauss-point computations of the reference's residualBulk, written once for a
// generic scalar type R.  The kernels instantiate R = double (device, built
// with -fmad=false so each operation is a separately rounded IEEE binary64
// operation in the reference's order); the operation counter instantiates an
// op-counting scalar on the host to obtain the algorithmic FLOP count.
//
// Terms that the reference evaluates with a third dimension are exact zeros
// in 2-D and are left out here; dropping an exact zero from a sum or a product
// changes no value, so the results still equal the reference's bit for bit.
#pragma once

#include <math.h>

#include <type_traits>

#include "vefem_internal.h"
#include "vefem_scalar.cuh"

#ifdef __CUDACC__
#define VF_HD __host__ __device__ __forceinline__
#else
#define VF_HD inline
#endif

namespace vefem {

// Divisions that share a divisor (the SQRT-form test-function terms divide by
// S11 + S22 and by Wi at every test node).  For FP64 on the device they use
// Markstein's method (P. Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): with
// r the correctly rounded reciprocal of y and q0 = RN(x r) within one ulp of
// x / y, the remainder e = x - q0 y is exact by FMA and RN(q0 + e r) is the
// correctly rounded quotient, i.e. the IEEE division's result, for operands
// and quotients in the normal range (the case here).  Other value types
// divide plainly.
template <class R>
VF_HD R recip_for_div(R y)
{
#ifdef __CUDA_ARCH__
    if constexpr (std::is_same<R, double>::value) return __drcp_rn(y);
#endif
    return y;   // unused by div_r below
}

template <class R>
VF_HD R div_r(R x, R y, R r)
{
#ifdef __CUDA_ARCH__
    if constexpr (std::is_same<R, double>::value) {
        const double q0 = x * r;
        if (q0 == 0.0) return q0;                   // keeps the sign of a zero quotient
        const double e = __fma_rn(-q0, y, x);
        return __fma_rn(e, r, q0);
    }
#endif
    (void)r;
    return x / y;
}


// FORM_T / FORM_SQRT and the specialisations SPEC_RE0 / SPEC_DF0 are in
// vefem_internal.h.
enum { L_PTT = 0, M_L_PTT = 1, E_PTT = 2, M_E_PTT = 3, FENE_CR = 4, FENE_P = 5, GIESEKUS = 6 };

// R is the scalar of state-dependent values, G the scalar of geometry values
// (basis derivatives, weights); the FP64 kernels use R = G = double, the
// exact-Jacobian kernels a dual number for R and float or double for G.

// ---------------------------------------------------------------------------
// Geometry of one Gauss point: basis2D (Element_Calculations_mod.F90:308-361),
// Helem of setStabilizationTerms (:718-727) and WET (Equations_mod.F90:85).
// x, y: the element's 9 node coordinates.  Outputs dFx, dFy, d2x, d2y [9].
template <class R>
struct GeoOut {
    R H2, WET, detJ;
};

template <class R, class B>
VF_HD GeoOut<R> geometry(const B *bfn_unused, const B *dfdc, const B *dfde, const B *d2c,
                        const B *d2e, const B *d2ce, B w, const R *x, const R *y, R *dFx,
                        R *dFy, R *d2x, R *d2y)
{
    (void)bfn_unused;
    R dxdc = 0.0, dydc = 0.0, dxde = 0.0, dyde = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        dxdc = dxdc + dfdc[n] * x[n];
        dydc = dydc + dfdc[n] * y[n];
        dxde = dxde + dfde[n] * x[n];
        dyde = dyde + dfde[n] * y[n];
    }
    GeoOut<R> g;
    g.detJ = dxdc * dyde - dxde * dydc;
    const R dcdx = dyde / g.detJ;
    const R dedx = -dydc / g.detJ;
    const R dcdy = -dxde / g.detJ;
    const R dedy = dxdc / g.detJ;
    R hs = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const R fx = (dcdx * dfdc[n] + dedx * dfde[n]);
        const R fy = (dcdy * dfdc[n] + dedy * dfde[n]);
        dFx[n] = fx;
        dFy[n] = fy;
        d2x[n] = (dcdx * dcdx) * d2c[n] + (dedx * dedx) * d2e[n] + (R)2.0 * dcdx * dedx * d2ce[n];
        d2y[n] = (dcdy * dcdy) * d2c[n] + (dedy * dedy) * d2e[n] + (R)2.0 * dcdy * dedy * d2ce[n];
        hs = hs + fx * fx + fy * fy;
    }
    const R helem = (R)1.0 / sqrt(hs);
    g.H2 = helem * helem;
    g.WET = w * fabs(g.detJ);
    return g;
}

// ---------------------------------------------------------------------------
// Interpolated unknowns at a Gauss point (setFlowUnknowns, :449-533).
template <class R>
struct Interp {
    R U1, U2, GU11, GU21, GU12, GU22, lap1, lap2, P, dPx, dPy;
    R S11, S12, S22, dS11x, dS11y, dS12x, dS12y, dS22x, dS22y;
};

// Gauss-point coefficients the test-function loop needs.
template <class R>
struct GpCoef {
    R U1, U2;
    R rc1, rc2;             // ReN * Convection(i)
    R P11, P12, P22;        // P_tot (P21 == P12 bit for bit)
    R M1, M2, Cont;         // Momentum, Continuity
    R tR;                   // tlsme * ReN
    R tlsme, tlsic, ntl, tlsce, tdcs, mag;
    R C11, C12, C21, C22;   // Con_EQ
    R S11, S12, S22, den;   // SQRT form: S and S11 + S22
    R rden, rWi;            // reciprocals for div_r (FP64 on the device; unused otherwise)
    R WiN, fT, omb;
    R dS11x, dS11y, dS12x, dS12y, dS22x, dS22y;
};

// interpolation from a state accessor V(pos), pos = inod*6 + ieq
template <class R, class View, class B>
VF_HD Interp<R> interpolate(const View &V, const B *bfn, const R *dFx, const R *dFy,
                            const R *d2x, const R *d2y)
{
    Interp<R> I;
    R u1 = 0.0, u2 = 0.0, g11 = 0.0, g21 = 0.0, g12 = 0.0, g22 = 0.0;
    R h11 = 0.0, h21 = 0.0, h12 = 0.0, h22 = 0.0, p = 0.0, px = 0.0, py = 0.0;
    R s11 = 0.0, s12 = 0.0, s22 = 0.0, a = 0.0, b = 0.0, c = 0.0, d = 0.0, e = 0.0, f = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const R t0 = V(n * 6 + 0), t1 = V(n * 6 + 1), t2 = V(n * 6 + 2);
        const R t3 = V(n * 6 + 3), t4 = V(n * 6 + 4), t5 = V(n * 6 + 5);
        const R bf = bfn[n], fx = dFx[n], fy = dFy[n], sx = d2x[n], sy = d2y[n];
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

// Interpolants of one field f (value, x/y gradients, x/y second derivatives)
// from a state accessor V(pos); the same sums, in the same order, as
// interpolate() forms for that field.  Written into a copy of the cached
// interpolants of the unperturbed state.
template <class R, class View>
VF_HD void interpolate_field(const View &V, int f, const double *bfn, const R *dFx, const R *dFy,
                             const R *d2x, const R *d2y, Interp<R> &I)
{
    R val = 0.0, gx = 0.0, gy = 0.0, hx = 0.0, hy = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const R t = V(n * 6 + f);
        val = val + t * bfn[n];
        gx = gx + t * dFx[n];
        gy = gy + t * dFy[n];
        hx = hx + t * d2x[n];
        hy = hy + t * d2y[n];
    }
    const R lap = hx + hy;
    I.U1 = f == 0 ? val : I.U1;
    I.GU11 = f == 0 ? gx : I.GU11;
    I.GU21 = f == 0 ? gy : I.GU21;
    I.lap1 = f == 0 ? lap : I.lap1;
    I.U2 = f == 1 ? val : I.U2;
    I.GU12 = f == 1 ? gx : I.GU12;
    I.GU22 = f == 1 ? gy : I.GU22;
    I.lap2 = f == 1 ? lap : I.lap2;
    I.P = f == 2 ? val : I.P;
    I.dPx = f == 2 ? gx : I.dPx;
    I.dPy = f == 2 ? gy : I.dPy;
    I.S11 = f == 3 ? val : I.S11;
    I.dS11x = f == 3 ? gx : I.dS11x;
    I.dS11y = f == 3 ? gy : I.dS11y;
    I.S12 = f == 4 ? val : I.S12;
    I.dS12x = f == 4 ? gx : I.dS12x;
    I.dS12y = f == 4 ? gy : I.dS12y;
    I.S22 = f == 5 ? val : I.S22;
    I.dS22x = f == 5 ? gx : I.dS22x;
    I.dS22y = f == 5 ? gy : I.dS22y;
}

// Strong form and stabilisation at a Gauss point:
// strongFormEquations (:537-573), setFlowKinematics (:605-634), the
// constitutive routines (Constitutive_Models_mod.F90, Constitutive_Models_SQRT_mod.F90),
// strongFormMomentum/Continuity (:658-697), setStabilizationTerms (:701-773).
// dotU[n] = U . grad(phi_n) is returned for reuse by the test-function loop
// (the reference computes the same product there).
template <int FORM, int SPEC = 0, class R, class G>
VF_HD GpCoef<R> gauss_point(const Interp<R> &I, const KParams &prm, R WiN, G H2, const G *dFx,
                            const G *dFy, R *dotU)
{
    typedef typename ScalarOf<R>::type S;
    GpCoef<R> g;
    const S BvN = (S)prm.BvN, ReN = (S)prm.ReN, VeN = (S)prm.VeN, DfN = (S)prm.DfN;
    const S omb = (S)1.0 - BvN;
    g.omb = omb;
    g.WiN = WiN;
    g.U1 = I.U1;
    g.U2 = I.U2;
    // setFlowKinematics, N = 2
    const R tr = I.GU11 + I.GU22;
    const R trh = tr / 2.0;
    const R gt11 = I.GU11 - trh, gt22 = I.GU22 - trh;   // GU_tr diagonal
    const R Gd11 = gt11 + gt11, Gd22 = gt22 + gt22;     // G_dot_tr
    const R Gd12 = I.GU12 + I.GU21;
    const R S11 = I.S11, S12 = I.S12, S22 = I.S22;
    g.S11 = S11; g.S12 = S12; g.S22 = S22;
    g.dS11x = I.dS11x; g.dS11y = I.dS11y; g.dS12x = I.dS12x; g.dS12y = I.dS12y;
    g.dS22x = I.dS22x; g.dS22y = I.dS22y;

    R f1, f2, f3, fT;
    R divT1, divT2, C11, C12, C21, C22, C33 = 0.0, ddT, ddS, ddC;
    // UCD convective part U . grad S (identical in both forms)
    const R u11 = I.U1 * I.dS11x + I.U2 * I.dS11y;
    const R u12 = I.U1 * I.dS12x + I.U2 * I.dS12y;
    const R u22 = I.U1 * I.dS22x + I.U2 * I.dS22y;
    if (FORM == FORM_T) {
        // strongFormConEQ (Constitutive_Models_mod.F90:55-92): T_ve = S, dTdXi = dSdXi
        const R trT = S11 + S22;
        R MDfDt = 0.0;
        if (prm.model == FENE_CR || prm.model == FENE_P) {
            // setFENEMaterialDerivative :272-311 (steady)
            const R dfx0 = I.dS11x + I.dS22x, dfy0 = I.dS11y + I.dS22y;
            const S den = (prm.model == FENE_P) ? VeN : (VeN - (S)2.0);
            const R dfx = (WiN / omb) * dfx0 / den;
            const R dfy = (WiN / omb) * dfy0 / den;
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
        const R term_I = (prm.model == FENE_P) ? MDfDt / fT : 0.0;
        // setStressTensor :344
        g.P11 = (S11 + BvN * Gd11) - I.P;
        g.P12 = S12 + BvN * Gd12;
        g.P22 = (S22 + BvN * Gd22) - I.P;
        // setUpperConvectedDerivativeT :315-331
        const R m1_11 = gt11 * S11 + I.GU21 * S12, m1_12 = gt11 * S12 + I.GU21 * S22;
        const R m1_21 = I.GU12 * S11 + gt22 * S12, m1_22 = I.GU12 * S12 + gt22 * S22;
        const R m2_11 = S11 * gt11 + S12 * I.GU21, m2_12 = S11 * I.GU12 + S12 * gt22;
        const R m2_21 = S12 * gt11 + S22 * I.GU21, m2_22 = S12 * I.GU12 + S22 * gt22;
        const R ucd11 = (u11 - m1_11) - m2_11, ucd12 = (u12 - m1_12) - m2_12;
        const R ucd21 = (u12 - m1_21) - m2_21, ucd22 = (u22 - m1_22) - m2_22;
        const R q11 = S11 * S11 + S12 * S12, q12 = S11 * S12 + S12 * S22;
        const R q22 = S12 * S12 + S22 * S22;
        const R fo = f1 * omb;
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
        const R Cc11 = S11 * S11 + S12 * S12, Cc12 = S11 * S12 + S12 * S22;
        const R Cc22 = S12 * S12 + S22 * S22;
        const R dC11x = (I.dS11x * S11 + I.dS12x * S12) + (S11 * I.dS11x + S12 * I.dS12x);
        const R dC12x = (I.dS11x * S12 + I.dS12x * S22) + (S11 * I.dS12x + S12 * I.dS22x);
        const R dC22x = (I.dS12x * S12 + I.dS22x * S22) + (S12 * I.dS12x + S22 * I.dS22x);
        const R dC11y = (I.dS11y * S11 + I.dS12y * S12) + (S11 * I.dS11y + S12 * I.dS12y);
        const R dC12y = (I.dS11y * S12 + I.dS12y * S22) + (S11 * I.dS12y + S12 * I.dS22y);
        const R dC22y = (I.dS12y * S12 + I.dS22y * S22) + (S12 * I.dS12y + S22 * I.dS22y);
        const R trC = Cc11 + Cc22;
        R g1 = 1.0, g2 = 1.0, dg1x = 0.0, dg1y = 0.0, dg2x = 0.0, dg2y = 0.0;
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
        const R rr = omb / WiN;
        const R T11 = rr * (g2 * Cc11 - g1), T12 = rr * (g2 * Cc12);
        const R T22 = rr * (g2 * Cc22 - g1), T33 = rr * (-g1);
        g.P11 = (T11 + BvN * Gd11) - I.P;
        g.P12 = T12 + BvN * Gd12;
        g.P22 = (T22 + BvN * Gd22) - I.P;
        const R dT11x = rr * ((dg2x * Cc11 + g2 * dC11x) - dg1x);
        const R dT12y = rr * (dg2y * Cc12 + g2 * dC12y);
        const R dT12x = rr * (dg2x * Cc12 + g2 * dC12x);
        const R dT22y = rr * ((dg2y * Cc22 + g2 * dC22y) - dg1y);
        divT1 = dT11x + dT12y;
        divT2 = dT12x + dT22y;
        // setUpperConvectedDerivativeSQRT :397-416 with WTensor2D :513-530
        const R den = S11 + S22;
        const R nW = (-(S11 * I.GU12) + S12 * (gt11 - gt22)) + S22 * I.GU21;
        const R W12 = nW / den;
        const R W21 = -W12;
        const R m1_11 = S11 * gt11 + S12 * I.GU21, m1_12 = S11 * I.GU12 + S12 * gt22;
        const R m1_21 = S12 * gt11 + S22 * I.GU21, m1_22 = S12 * I.GU12 + S22 * gt22;
        const R ucd11 = (u11 - m1_11) - W12 * S12, ucd12 = (u12 - m1_12) - W12 * S22;
        const R ucd21 = (u12 - m1_21) - W21 * S11, ucd22 = (u22 - m1_22) - W21 * S12;
        // setSInverse :459-479 (inverseTensor2D, Tools_mod.F90:129-146)
        const R det = S11 * S22 - S12 * S12;
        const R SI11 = S22 / det, SI12 = (-S12) / det, SI22 = S11 / det;
        const R s3_11 = S11 * Cc11 + S12 * Cc12, s3_12 = S11 * Cc12 + S12 * Cc22;
        const R s3_21 = S12 * Cc11 + S22 * Cc12, s3_22 = S12 * Cc12 + S22 * Cc22;
        C11 = WiN * ucd11 + ((f3 * s3_11 + f2 * S11) - f1 * SI11) / 2.0;
        C12 = WiN * ucd12 + ((f3 * s3_12 + f2 * S12) - f1 * SI12) / 2.0;
        C21 = WiN * ucd21 + ((f3 * s3_21 + f2 * S12) - f1 * SI12) / 2.0;
        C22 = WiN * ucd22 + ((f3 * s3_22 + f2 * S22) - f1 * SI22) / 2.0;
        ddT = (((T11 * T11 + T12 * T12) + T12 * T12) + T22 * T22) + T33 * T33;
        ddS = ((S11 * S11 + S12 * S12) + S12 * S12) + S22 * S22;
        ddC = ((Cc11 * Cc11 + Cc12 * Cc12) + Cc12 * Cc12) + Cc22 * Cc22;
        g.den = den;
        g.rden = recip_for_div(den);
        g.rWi = recip_for_div(WiN);
    }
    g.fT = fT;
    g.C11 = C11; g.C12 = C12; g.C21 = C21; g.C22 = C22;
    // strongFormMomentum :658-683, strongFormContinuity :687-697
    const R divP1 = (-I.dPx + divT1) + BvN * I.lap1;
    const R divP2 = (-I.dPy + divT2) + BvN * I.lap2;
    const R conv1 = I.U1 * I.GU11 + I.U2 * I.GU21;
    const R conv2 = I.U1 * I.GU12 + I.U2 * I.GU22;
    if (SPEC & SPEC_RE0) {
        g.rc1 = 0.0;
        g.rc2 = 0.0;
        g.M1 = -divP1;
        g.M2 = -divP2;
    } else {
        g.rc1 = ReN * conv1;
        g.rc2 = ReN * conv2;
        g.M1 = g.rc1 - divP1;
        g.M2 = g.rc2 - divP2;
    }
    g.Cont = tr;
    // setStabilizationTerms :701-773
    R tsugn = 0.0;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const R du = I.U1 * dFx[n] + I.U2 * dFy[n];
        dotU[n] = du;
        tsugn = tsugn + fabs(du);
    }
    const R ddG = ((Gd11 * Gd11 + Gd12 * Gd12) + Gd12 * Gd12) + Gd22 * Gd22;
    const R r = omb / WiN;
    R Ha = sqrt(r * r + 0.5 * ddT);
    Ha = Ha / sqrt(1.0 + 0.5 * ddG);
    const R a3 = BvN / H2, a4 = Ha / H2;
    R tlsme;
    if (SPEC & SPEC_RE0) {
        tlsme = a3 * a3 + a4 * a4;
    } else {
        const R a1 = ReN / (S)prm.dt, a2 = ReN * tsugn;
        tlsme = a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4;
    }
    tlsme = 1.0 / sqrt(tlsme);
    g.tlsme = tlsme;
    g.tlsic = H2 / tlsme;
    if (!(SPEC & SPEC_RE0)) g.tR = tlsme * ReN;
    R tdcs = 0.5 * ddS;
    if (FORM == FORM_T) tdcs = tdcs + r * r;
    tdcs = H2 / sqrt(tdcs);
    if (DfN > (S)1.0e-12) tdcs = 0.0;
    g.tdcs = tdcs;
    R mag = (((C11 * C11 + C12 * C21) + C21 * C12) + C22 * C22) + C33 * C33;
    mag = sqrt(0.5 * mag);
    g.mag = mag;
    const R b1 = WiN / (S)prm.dt, b2 = WiN * tsugn, b3 = WiN * sqrt(0.5 * ddG), b4 = f2;
    const R b5 = f3 * sqrt(0.5 * ddC), b6 = tdcs * mag / H2;
    R tlsce = b1 * b1 + b2 * b2 + b3 * b3 + b4 * b4 + b5 * b5 + b6 * b6;
    if (!(SPEC & SPEC_DF0)) {
        const R b7 = DfN / H2;
        tlsce = tlsce + b7 * b7;
    }
    tlsce = 1.0 / sqrt(tlsce);
    g.tlsce = tlsce;
    g.ntl = -tlsce;
    return g;
}

// Weak-form terms of one test node n (momentumMain(SQRT), continuityBulkMain,
// stressesBulkMain(SQRT), Residuals_mod.F90:44-157, 295-490) times WET.
template <int FORM, int SPEC = 0, class R, class B, class G, class Out>
VF_HD void test_node(const GpCoef<R> &g, const KParams &prm, B bifn, G fx, G fy, R du,
                     G WET, Out *out)
{
    typedef typename ScalarOf<R>::type S;
    const R DfN = (S)prm.DfN;
    // momentum
    R lsme1, lsme2;
    if (!(SPEC & SPEC_RE0)) {
        const R lme = g.tR * du;
        lsme1 = lme * g.M1;
        lsme2 = lme * g.M2;
    }
    const R lsic1 = (g.tlsic * fx) * g.Cont, lsic2 = (g.tlsic * fy) * g.Cont;
    R lsce1, lsce2;
    if (FORM == FORM_T) {
        // LSCEMomentumT :191-219 with doubleDotProduct (A:B^T)
        const R lx = g.ntl * fx, ly = g.ntl * fy;
        lsce1 = lx * g.C11 + ly * g.C21;
        lsce2 = lx * g.C12 + ly * g.C22;
    } else {
        // LSCEMomentumSQRT :388-433
        const R S11 = g.S11, S12 = g.S12, S22 = g.S22;
        const R m1a = S11 * fx + S12 * fy;   // (S . grad phi)_1
        const R m1b = S12 * fx + S22 * fy;   // (S . grad phi)_2
        const R wa = div_r(m1b, g.den, g.rden);          // W12 for i = 1
        const R wb = -div_r(m1a, g.den, g.rden);         // W12 for i = 2
        const R k = g.tlsce;
        const R omb = g.omb, Wi = g.WiN;
        // i = 1: GU_lsce column 1 = grad phi
        R u11 = -m1a - wa * S12, u12 = -(wa * S22);
        R u21 = -m1b - (-wa) * S11, u22 = -((-wa) * S12);
        const R rW = g.rWi;
        R l11 = div_r(k * u11 * omb, Wi, rW), l12 = div_r(k * u12 * omb, Wi, rW);
        R l21 = div_r(k * u21 * omb, Wi, rW), l22 = div_r(k * u22 * omb, Wi, rW);
        lsce1 = ((l11 * g.C11 + l12 * g.C21) + l21 * g.C12) + l22 * g.C22;
        // i = 2: GU_lsce column 2 = grad phi
        u11 = -(wb * S12);
        u12 = -m1a - wb * S22;
        u21 = -((-wb) * S11);
        u22 = -m1b - (-wb) * S12;
        l11 = div_r(k * u11 * omb, Wi, rW); l12 = div_r(k * u12 * omb, Wi, rW);
        l21 = div_r(k * u21 * omb, Wi, rW); l22 = div_r(k * u22 * omb, Wi, rW);
        lsce2 = ((l11 * g.C11 + l12 * g.C21) + l21 * g.C12) + l22 * g.C22;
    }
    const R pd1 = g.P11 * fx + g.P12 * fy;
    const R pd2 = g.P12 * fx + g.P22 * fy;
    R t0, t1;
    if (SPEC & SPEC_RE0) {
        t0 = (pd1 + lsic1) + lsce1;
        t1 = (pd2 + lsic2) + lsce2;
    } else {
        t0 = (((g.rc1 * bifn + pd1) + lsme1) + lsic1) + lsce1;
        t1 = (((g.rc2 * bifn + pd2) + lsme2) + lsic2) + lsce2;
    }
    // continuity
    const R t2 = g.Cont * bifn + g.tlsme * (fx * g.M1 + fy * g.M2);
    // stresses (j,k) = (1,1), (1,2), (2,2)
    const R gd11 = g.dS11x * fx + g.dS11y * fy;
    const R gd12 = g.dS12x * fx + g.dS12y * fy;
    const R gd22 = g.dS22x * fx + g.dS22y * fy;
    R ls11 = -fx * g.M1;
    R ls12 = -fy * g.M1 - fx * g.M2;
    R ls22 = -fy * g.M2;
    R lce;
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
    R t3, t4, t5;
    if (SPEC & SPEC_DF0) {
        t3 = ((g.C11 * bifn + ls11) + lce * g.C11) + (g.tdcs * gd11) * g.mag;
        t4 = ((g.C12 * bifn + ls12) + lce * g.C12) + (g.tdcs * gd12) * g.mag;
        t5 = ((g.C22 * bifn + ls22) + lce * g.C22) + (g.tdcs * gd22) * g.mag;
    } else {
        t3 = (((g.C11 * bifn + DfN * gd11) + ls11) + lce * g.C11) + (g.tdcs * gd11) * g.mag;
        t4 = (((g.C12 * bifn + DfN * gd12) + ls12) + lce * g.C12) + (g.tdcs * gd12) * g.mag;
        t5 = (((g.C22 * bifn + DfN * gd22) + ls22) + lce * g.C22) + (g.tdcs * gd22) * g.mag;
    }
    out[0] = t0 * WET;
    out[1] = t1 * WET;
    out[2] = t2 * WET;
    out[3] = t3 * WET;
    out[4] = t4 * WET;
    out[5] = t5 * WET;
}


}  // namespace vefem
