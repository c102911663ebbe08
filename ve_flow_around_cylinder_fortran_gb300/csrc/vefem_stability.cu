// Linear-stability assembly: the A and B matrices of the generalised
// eigenproblem for spanwise-periodic 3-D perturbations (Neq = 10 per node:
// Ux, Uy, Uz, P, Txx, Txy, Tyy, Txz, Tyz, Tzz) of a steady 2-D base state,
// for many wavenumbers at once (setEquationsBulkStability,
// Equations_Stability_mod.F90:20-226; T form).
//
// The perturbation residual is linear in the perturbation, with the base
// state's quantities as coefficients, and at a Gauss point its weak-form
// term for test node i is linear in the test function's (phi, dphi/dx,
// dphi/dy):  TERM(i, e) = sum_k psi_k(i) c_ek(q).  The coefficients c depend
// linearly on 33 interpolated perturbation quantities q (velocity: value,
// x/y gradient, Laplacian; pressure and the six stresses: value, x/y
// gradient); the z-derivatives follow from the values and the wavenumber K
// (setExtraFlowUnknownsStability, Element_Calculations_Stability_mod.F90:280-311).
// The element matrices are therefore
//     A(i,e; j,f) = sum_gp WET sum_k psi_k(i) sum_s D[gp][q(f,s)][e][k] chi_s(j)
// with D = dc/dq obtained by evaluating c at unit q.  A is a quadratic
// polynomial in K and B does not depend on it, so the kernel builds the
// element blocks of B and of A at K = 0, +1, -1 once, and the scatter forms
// A(K) = A0 + K (A+ - A-)/2 + K^2 ((A+ + A-)/2 - A0) for every requested
// wavenumber while it sums the element blocks in element order.
//
// FP64 throughout.  Base quantities per Gauss point follow strongFormEquations
// with the stability problem's dimension N = 3 (traceless kinematics) and
// setStabilizationTerms; the perturbation physics restates
// setFlowQuantitiesStability, strongFormConEQ_Stability (L-PTT, m-L-PTT,
// e-PTT, m-e-PTT, Giesekus), strongFormMomentumStability and the terms of
// momentumStabilityT, momentumStability3D, continuityStability and
// stressStabilityT (Residuals_Stability_mod.F90:34-188).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "vefem.h"
#include "vefem_ctx.h"
#include "vefem_internal.h"
#include "vefem_physics.cuh"

namespace vefem {

namespace {

constexpr int ST_NEQ = 10;
constexpr int ST_NQ = 33;          // perturbation quantities
constexpr int ST_THREADS = 256;
constexpr int ST_BLK = 8100;       // 90 x 90 element block

__constant__ double s_w[9];
__constant__ double s_bfn[9][9], s_dfdc[9][9], s_dfde[9][9], s_d2c[9][9], s_d2e[9][9], s_d2ce[9][9];

// base quantities a Gauss point needs (StabBase) -- 3x3 tensors as the reference holds them
struct StabBase {
    double U[3];
    double GU[3][3], GUT[3][3], G_dot[3][3];
    double S[3][3], dT[3][3][3];
    double CE[3][3];                   // Con_EQ
    double f[3], g[2], fT;
    double tlsme, tlsic, tlsce, tdcs, mag;
    double WET;
};

__device__ __forceinline__ double tr3(const double A[3][3]) { return A[0][0] + A[1][1] + A[2][2]; }

// doubleDotProduct (Tools_mod.F90:262-280): sum_ij A(i,j) B(j,i)
__device__ __forceinline__ double ddot(const double A[3][3], const double B[3][3])
{
    double s = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) s = s + A[i][j] * B[j][i];
    return s;
}

__device__ __forceinline__ void mm3(const double A[3][3], const double B[3][3], double C[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s = s + A[i][k] * B[k][j];
            C[i][j] = s;
        }
}

// stress component of unknown i - istart (getStressComponent, Tools_mod.F90:769-793)
__device__ __forceinline__ void stress_jk(int c, int &j, int &k)
{
    const int J[6] = {0, 0, 1, 0, 1, 2}, K[6] = {0, 1, 1, 2, 2, 2};
    j = J[c];
    k = K[c];
}

// Base state at Gauss point ig of an element: setFlowUnknownsStability on
// TEMP_TL_b, strongFormEquations(Problem_Stability) (N = 3), setStabilizationTerms.
__device__ void stab_base(const KParams &p, const double *tlb /* [9][10] */, const double *dFx,
                          const double *dFy, const double *d2x, const double *d2y, double H2,
                          double WET, int ig, StabBase &b)
{
    const double WiN = p.WiN, BvN = p.BvN, VeN = p.VeN, ReN = p.ReN, DfN = p.DfN, dt = p.dt;
    double GU[3][3] = {}, G2U[3][3] = {}, U[3] = {}, dP[3] = {}, P = 0.0;
    double S[3][3] = {}, dS[3][3][3] = {};
    for (int i = 0; i < 3; i++) {
        double u = 0.0, gx = 0.0, gy = 0.0, hx = 0.0, hy = 0.0, px = 0.0, py = 0.0;
        for (int n = 0; n < 9; n++) {
            const double t = tlb[n * ST_NEQ + i];
            u = u + t * s_bfn[ig][n];
            gx = gx + t * dFx[n];
            gy = gy + t * dFy[n];
            hx = hx + t * d2x[n];
            hy = hy + t * d2y[n];
        }
        U[i] = u;
        GU[0][i] = gx;
        GU[1][i] = gy;
        G2U[0][i] = hx;
        G2U[1][i] = hy;
    }
    {
        double pv = 0.0, px = 0.0, py = 0.0;
        for (int n = 0; n < 9; n++) {
            const double t = tlb[n * ST_NEQ + 3];
            pv = pv + t * s_bfn[ig][n];
            px = px + t * dFx[n];
            py = py + t * dFy[n];
        }
        P = pv;
        dP[0] = px;
        dP[1] = py;
    }
    for (int c = 0; c < 6; c++) {
        int j, k;
        stress_jk(c, j, k);
        double v = 0.0, gx = 0.0, gy = 0.0;
        for (int n = 0; n < 9; n++) {
            const double t = tlb[n * ST_NEQ + 4 + c];
            v = v + t * s_bfn[ig][n];
            gx = gx + t * dFx[n];
            gy = gy + t * dFy[n];
        }
        S[j][k] = v;
        S[k][j] = v;
        dS[j][k][0] = gx;
        dS[j][k][1] = gy;
        dS[k][j][0] = gx;
        dS[k][j][1] = gy;
    }
    // setFlowKinematics, N = 3
    double GUT[3][3], Gd[3][3], GUtr[3][3], GUTtr[3][3], Gdtr[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) GUT[i][j] = GU[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Gd[i][j] = GU[i][j] + GUT[i][j];
    const double trg = tr3(GU);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) GUtr[i][j] = GU[i][j] - trg * (i == j ? 1.0 : 0.0) / 3.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) GUTtr[i][j] = GUtr[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Gdtr[i][j] = GUtr[i][j] + GUTtr[i][j];
    // conEQ_* (Constitutive_Models_mod.F90:96-268), models restated for stability
    const double trT = tr3(S);
    const bool fene = p.model == FENE_CR || p.model == FENE_P;
    double fT = 1.0, f0 = 1.0, f1 = 1.0, f2 = 0.0, g0 = 1.0, g1 = 1.0, termI = 0.0;
    if (p.model == L_PTT || p.model == M_L_PTT) {
        fT = 1.0 + (VeN * WiN * trT) / (1.0 - BvN);
    } else if (p.model == E_PTT || p.model == M_E_PTT) {
        fT = exp(VeN * WiN * trT / (1.0 - BvN));
    } else if (p.model == FENE_CR) {   // N = 2, the base problem's dimension
        fT = 1.0 + ((WiN * trT / (1.0 - BvN))) / (VeN - 2.0);
    } else if (p.model == FENE_P) {
        fT = 1.0 + (WiN * trT / (1.0 - BvN)) / VeN;
    } else {  // GIESEKUS
        fT = VeN * WiN / (1.0 - BvN);
    }
    if (p.model == GIESEKUS) {
        f2 = fT;
    } else if (p.model == M_L_PTT || p.model == M_E_PTT) {
        f0 = fT; f1 = fT; g0 = fT; g1 = fT;
    } else if (fene) {
        // setFENEMaterialDerivative (steady): U . grad f_T from the trace of grad T
        double df[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) df[c] = df[c] + dS[i][i][c];
        const double den = p.model == FENE_P ? VeN : (VeN - 2.0);
        for (int c = 0; c < 3; c++) df[c] = (WiN / (1.0 - BvN)) * df[c] / den;
        double MD = 0.0;
        for (int i = 0; i < 3; i++) MD = MD + U[i] * df[i];
        f1 = fT - (WiN * MD / fT);
        if (p.model == FENE_CR) {
            f0 = fT; g0 = fT; g1 = fT;
        } else {
            g1 = fT;
            termI = MD / fT;
        }
    } else {
        f1 = fT;
    }
    // upper-convected derivative (steady) and Con_EQ
    double UCD[3][3] = {}, M1[3][3], M2[3][3], T2[3][3];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] + U[k] * dS[i][j][k];
    mm3(GUTtr, S, M1);
    mm3(S, GUtr, M2);
    mm3(S, S, T2);
    double CE[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const double ucd = UCD[i][j] - M1[i][j] - M2[i][j];
            double c = WiN * ucd + f2 * T2[i][j];
            c = c + f1 * S[i][j];
            c = c - f0 * (1.0 - BvN) * (Gdtr[i][j] + termI * (i == j ? 1.0 : 0.0));
            CE[i][j] = c;
        }
    // setStabilizationTerms
    double tsugn = 0.0;
    for (int n = 0; n < 9; n++) tsugn = tsugn + fabs(U[0] * dFx[n] + U[1] * dFy[n]);
    const double ddT = ddot(S, S), ddG = ddot(Gdtr, Gdtr);
    double Ha = sqrt(((1.0 - BvN) / WiN) * ((1.0 - BvN) / WiN) + 0.5 * ddT);
    Ha = Ha / sqrt(1.0 + 0.5 * ddG);
    const double t1 = ReN / dt, t2 = ReN * tsugn, t3 = BvN / H2, t4 = Ha / H2;
    double tlsme = t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4;
    tlsme = 1.0 / sqrt(tlsme);
    double tdcs = 0.5 * ddot(S, S);
    tdcs = tdcs + ((1.0 - BvN) / WiN) * ((1.0 - BvN) / WiN);
    tdcs = H2 / sqrt(tdcs);
    if (DfN > 1.0e-12) tdcs = 0.0;
    double mag = sqrt(0.5 * ddot(CE, CE));
    const double s1 = WiN / dt, s2 = WiN * tsugn, s3 = WiN * sqrt(0.5 * ddG), s4 = f1;
    const double s5 = f2 * sqrt(0.5 * ddT), s6 = tdcs * mag / H2, s7 = DfN / H2;
    double tlsce = s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4 + s5 * s5 + s6 * s6 + s7 * s7;
    tlsce = 1.0 / sqrt(tlsce);

    for (int i = 0; i < 3; i++) {
        b.U[i] = U[i];
        for (int j = 0; j < 3; j++) {
            b.GU[i][j] = GU[i][j];
            b.GUT[i][j] = GUT[i][j];
            b.G_dot[i][j] = Gd[i][j];
            b.S[i][j] = S[i][j];
            b.CE[i][j] = CE[i][j];
            for (int k = 0; k < 3; k++) b.dT[i][j][k] = dS[i][j][k];
        }
    }
    b.f[0] = f0; b.f[1] = f1; b.f[2] = f2; b.g[0] = g0; b.g[1] = g1; b.fT = fT;
    b.tlsme = tlsme;
    b.tlsic = H2 / tlsme;
    b.tlsce = tlsce;
    b.tdcs = tdcs;
    b.mag = mag;
    b.WET = WET;
    (void)P; (void)dP; (void)G2U;
}

// Coefficients c_a[e][k], c_b[e][k] (k: phi, dphi/dx, dphi/dy) of the
// perturbation's weak-form terms at one Gauss point for unit quantity q.
__device__ void stab_coef(const KParams &p, const StabBase &b, double K, int kz, int q,
                          double ca[ST_NEQ][3], double cb[ST_NEQ][3])
{
    const double WiN = p.WiN, BvN = p.BvN, ReN = p.ReN, DfN = p.DfN, VeN = p.VeN;
    double U[3] = {}, GU[3][3] = {}, G2U[3][3] = {}, P = 0.0, dP[3] = {};
    double S[3][3] = {}, dT[3][3][3] = {};
    // unit interpolant q: velocity i: value, d/dx, d/dy, Laplacian (x and y parts summed)
    if (q < 12) {
        const int i = q / 4, s = q % 4;
        if (s == 0) U[i] = 1.0;
        else if (s == 1) GU[0][i] = 1.0;
        else if (s == 2) GU[1][i] = 1.0;
        else G2U[0][i] = 1.0;
    } else if (q < 15) {
        const int s = q - 12;
        if (s == 0) P = 1.0;
        else dP[s - 1] = 1.0;
    } else {
        const int c = (q - 15) / 3, s = (q - 15) % 3;
        int j, k;
        stress_jk(c, j, k);
        if (s == 0) {
            S[j][k] = 1.0;
            S[k][j] = 1.0;
        } else {
            dT[j][k][s - 1] = 1.0;
            dT[k][j][s - 1] = 1.0;
        }
    }
    if (kz) {   // setExtraFlowUnknownsStability, real split, N = z
        GU[2][0] = -K * U[0];
        GU[2][1] = -K * U[1];
        GU[2][2] = K * U[2];
        dP[2] = -K * P;
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) dT[a][c][2] = -K * S[a][c];
        dT[0][2][2] = K * S[0][2];
        dT[2][0][2] = dT[0][2][2];
        dT[1][2][2] = K * S[1][2];
        dT[2][1][2] = dT[1][2][2];
        for (int i = 0; i < 3; i++) G2U[2][i] = -(K * K) * U[i];
    }
    // setFlowKinematics
    double GUT[3][3], Gd[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) GUT[i][j] = GU[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Gd[i][j] = GU[i][j] + GUT[i][j];
    // conEQ_*_Stability (Constitutive_Models_Stability_mod.F90:96-289)
    const double trT = tr3(S);
    const bool fene = p.model == FENE_CR || p.model == FENE_P;
    double fT = 0.0, f0 = 0.0, f1 = 0.0, termI = 0.0, termIt = 0.0;
    if (p.model == L_PTT || p.model == M_L_PTT) fT = VeN * WiN * trT / (1.0 - BvN);
    else if (p.model == E_PTT || p.model == M_E_PTT) fT = b.fT * VeN * WiN * trT / (1.0 - BvN);
    else if (p.model == FENE_CR) fT = (WiN * trT / (1.0 - BvN)) / (VeN - 2.0);
    else if (p.model == FENE_P) fT = (WiN * trT / (1.0 - BvN)) / VeN;
    if (p.model == M_L_PTT || p.model == M_E_PTT || p.model == FENE_CR) f0 = fT;
    if (p.model != GIESEKUS) f1 = fT;
    if (fene) {
        // setFENEMaterialDerivativeStability (:294-328)
        double dfb[3] = {0.0, 0.0, 0.0}, dfd[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) {
                dfb[c] = dfb[c] + b.dT[i][i][c];
                dfd[c] = dfd[c] + dT[i][i][c];
            }
        const double den = p.model == FENE_P ? VeN : (VeN - 2.0);
        for (int c = 0; c < 3; c++) {
            dfb[c] = (WiN / (1.0 - BvN)) * dfb[c] / den;
            dfd[c] = (WiN / (1.0 - BvN)) * dfd[c] / den;
        }
        double MD = 0.0;
        for (int i = 0; i < 3; i++) {
            const double term = ((b.fT) * dfd[i] - fT * dfb[i]) / (b.fT);
            MD = MD + U[i] * dfb[i] + b.U[i] * term;
        }
        f1 = fT - WiN * MD / (b.fT);
        if (p.model == FENE_P) {
            termI = MD / (b.fT);
            termIt = -(1.0 - BvN) * fT / (b.fT);
        }
    }
    // setStressTensorStability: P_tot (C_Tensor of the perturbation is not used below)
    double Pt[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Pt[i][j] = S[i][j] + BvN * Gd[i][j] - P * (i == j ? 1.0 : 0.0);
    // setUCDStability
    double UCD[3][3] = {}, M1[3][3], M2[3][3], M3[3][3], M4[3][3];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] + b.U[k] * dT[i][j][k] + U[k] * b.dT[i][j][k];
    mm3(b.GUT, S, M1);
    mm3(GUT, b.S, M2);
    mm3(b.S, GU, M3);
    mm3(S, b.GU, M4);
    double SbSd[3][3], SdSb[3][3], SbSb[3][3], CE[3][3];
    mm3(b.S, S, SbSd);
    mm3(S, b.S, SdSb);
    mm3(b.S, b.S, SbSb);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const double ucd = UCD[i][j] - M1[i][j] - M2[i][j] - M3[i][j] - M4[i][j];
            const double tT = b.f[2] * (SbSd[i][j] + SdSb[i][j]) + 0.0 * SbSb[i][j] + f1 * b.S[i][j]
                              + b.f[1] * S[i][j];
            const double tG = b.f[0] * Gd[i][j] + f0 * b.G_dot[i][j];
            CE[i][j] = WiN * ucd + tT - (1.0 - BvN) * (tG + termI * (i == j ? 1.0 : 0.0));
        }
    // strongFormMomentumStability
    double Mom[3], mt[3];
    for (int i = 0; i < 3; i++) {
        double divT = 0.0;
        for (int j = 0; j < 3; j++) divT = divT + dT[j][i][j];
        const double divP = -dP[i] + divT + BvN * (G2U[0][i] + G2U[1][i] + G2U[2][i]);
        double c1 = 0.0, c2 = 0.0;
        for (int k = 0; k < 3; k++) c1 = c1 + b.U[k] * GU[k][i];
        for (int k = 0; k < 3; k++) c2 = c2 + U[k] * b.GU[k][i];
        Mom[i] = ReN * (c1 + c2) - divP;
        mt[i] = ReN * U[i];
    }
    const double Cont = tr3(GU);
    const double magd = ddot(b.CE, CE) / (2.0 * b.mag + 1.0e-12);
    double ceqt[3][3];     // Con_EQ_time (strongFormConEQ_Stability :85-93)
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double c = WiN * S[i][j];
            if (fene) c = c - WiN * fT * b.S[i][j] / (b.fT);
            ceqt[i][j] = c + termIt * (i == j ? 1.0 : 0.0);
        }
    double conv[3];
    for (int i = 0; i < 3; i++) {
        double c1 = 0.0, c2 = 0.0;
        for (int k = 0; k < 3; k++) c1 = c1 + b.U[k] * GU[k][i];
        for (int k = 0; k < 3; k++) c2 = c2 + U[k] * b.GU[k][i];
        conv[i] = c1 + c2;
    }
    // momentumStabilityT + momentumStability3D
    const double lme[2] = {b.tlsme * ReN * b.U[0], b.tlsme * ReN * b.U[1]};   // LSMEMomentum per dphi
    for (int i = 0; i < 3; i++) {
        const double k3 = (i == 2) ? -K : K;
        ca[i][0] = ReN * conv[i] - k3 * Pt[i][2];
        cb[i][0] = mt[i];
        for (int c = 0; c < 2; c++) {
            ca[i][1 + c] = Pt[i][c] + lme[c] * Mom[i] + (i == c ? b.tlsic * Cont : 0.0)
                           - b.tlsce * CE[c][i];
            cb[i][1 + c] = lme[c] * mt[i] - b.tlsce * ceqt[c][i];
        }
    }
    // continuityStability
    ca[3][0] = Cont;
    cb[3][0] = 0.0;
    for (int c = 0; c < 2; c++) {
        ca[3][1 + c] = b.tlsme * Mom[c];
        cb[3][1 + c] = b.tlsme * mt[c];
    }
    // stressStabilityT
    for (int cc = 0; cc < 6; cc++) {
        int j, k;
        stress_jk(cc, j, k);
        const int e = 4 + cc;
        ca[e][0] = CE[j][k];
        cb[e][0] = ceqt[j][k];
        for (int c = 0; c < 2; c++) {
            double lm = -(k == c ? Mom[j] : 0.0);
            double lt = -(k == c ? mt[j] : 0.0);
            if (j != k) {
                lm = lm - (j == c ? Mom[k] : 0.0);
                lt = lt - (j == c ? mt[k] : 0.0);
            }
            const double lce = b.tlsce * WiN * b.U[c];
            const double dcs = b.tdcs * b.dT[j][k][c];
            ca[e][1 + c] = DfN * dT[j][k][c] + b.tlsme * lm * (1.0 - BvN) + lce * CE[j][k] + dcs * magd;
            cb[e][1 + c] = b.tlsme * lt * (1.0 - BvN) + lce * ceqt[j][k];
        }
    }
    // TERM_RES_b = -TERM_RES_b
    for (int e = 0; e < ST_NEQ; e++)
        for (int c = 0; c < 3; c++) cb[e][c] = -cb[e][c];
}

struct StabArgs {
    int nel, nnodes;
    const int32_t *conn;
    const double *xy;
    const double *TLb;      // [10][nnodes] embedded base state
    double *es;             // [nel][4][ST_BLK]: B, A(0), A(+1), A(-1), block layout
    int kz;
};

// quantity index of field f, basis component s (0 value, 1 d/dx, 2 d/dy, 3 Laplacian)
__device__ __forceinline__ int st_q(int f, int s)
{
    return f < 3 ? f * 4 + s : (f == 3 ? 12 + s : 15 + (f - 4) * 3 + s);
}

constexpr int ST_JCH = 3;                                            // test nodes per chunk
constexpr int ST_CH_OUT = ST_JCH * 900;                              // outputs per chunk (2700)
constexpr int ST_PER_T = (ST_CH_OUT + ST_THREADS - 1) / ST_THREADS;  // outputs per thread (11)
constexpr int ST_A2 = ST_NQ + 1;                                     // row stride of A2

// Shared memory: D and DB [9][33][10][3] coefficient derivatives (A at one K
// and, from the same evaluations at K = 0, B), A2 [30][ST_A2] the test-side
// contraction of one Gauss point for one chunk of three test nodes, and the
// base quantities of the 9 Gauss points.
__host__ __device__ constexpr size_t st_smem_doubles()
{
    return (size_t)2 * 9 * ST_NQ * ST_NEQ * 3 + (size_t)ST_JCH * ST_NEQ * ST_A2;
}

__global__ void __launch_bounds__(ST_THREADS)
k_stability(const StabArgs a, const KParams prm)
{
    extern __shared__ __align__(16) double sm[];
    double *D = sm;                                   // [9][33][10][3]
    double *DB = D + 9 * ST_NQ * ST_NEQ * 3;          // [9][33][10][3]
    double *A2 = DB + 9 * ST_NQ * ST_NEQ * 3;         // [30][ST_A2]
    StabBase *base = reinterpret_cast<StabBase *>(A2 + ST_JCH * ST_NEQ * ST_A2);
    __shared__ double s_tlb[9 * ST_NEQ];
    __shared__ double s_dFx[9][9], s_dFy[9][9], s_lap[9][9], s_H2[9], s_W[9];
    __shared__ double s_d2x[9][9], s_d2y[9][9];
    const int t = threadIdx.x;
    for (int e = blockIdx.x; e < a.nel; e += gridDim.x) {
        if (t < 9 * ST_NEQ) {
            const int n = t / ST_NEQ, f = t % ST_NEQ;
            s_tlb[t] = a.TLb[(size_t)f * a.nnodes + a.conn[n * a.nel + e]];
        } else if (t >= 96 && t < 105) {
            const int ig = t - 96;
            double x[9], y[9], fx[9], fy[9], sx[9], sy[9];
            for (int n = 0; n < 9; n++) {
                const int gn = a.conn[n * a.nel + e];
                x[n] = a.xy[gn];
                y[n] = a.xy[a.nnodes + gn];
            }
            auto go = geometry(s_bfn[ig], s_dfdc[ig], s_dfde[ig], s_d2c[ig], s_d2e[ig], s_d2ce[ig],
                               s_w[ig], x, y, fx, fy, sx, sy);
            for (int n = 0; n < 9; n++) {
                s_dFx[ig][n] = fx[n];
                s_dFy[ig][n] = fy[n];
                s_d2x[ig][n] = sx[n];
                s_d2y[ig][n] = sy[n];
                s_lap[ig][n] = sx[n] + sy[n];
            }
            s_H2[ig] = go.H2;
            s_W[ig] = go.WET;
        }
        __syncthreads();
        if (t < 9)
            stab_base(prm, s_tlb, s_dFx[t], s_dFy[t], s_d2x[t], s_d2y[t], s_H2[t], s_W[t], t, base[t]);
        __syncthreads();
        double *out = a.es + (size_t)e * 4 * ST_BLK;
        // element block m: 0 B (K = 0), 1 A(0), 2 A(+1), 3 A(-1); layout
        // ((jnod*9 + inod)*10 + jeq)*10 + ieq: row (jnod, jeq) = equation of test node
        // jnod, column (inod, ieq) = unknown of trial node inod.  The K = 0
        // evaluations give both B and A(0).
        for (int m = 0; m < 4; m++) {
            const double K = m == 2 ? 1.0 : (m == 3 ? -1.0 : 0.0);
            if (m != 1) {
                for (int w = t; w < 9 * ST_NQ; w += ST_THREADS) {
                    const int gp = w / ST_NQ, q = w % ST_NQ;
                    double ca[ST_NEQ][3], cb[ST_NEQ][3];
                    stab_coef(prm, base[gp], K, a.kz, q, ca, cb);
                    double *da = D + (size_t)w * ST_NEQ * 3, *db = DB + (size_t)w * ST_NEQ * 3;
                    for (int e2 = 0; e2 < ST_NEQ; e2++)
                        for (int c = 0; c < 3; c++) {
                            da[e2 * 3 + c] = ca[e2][c];
                            if (m == 0) db[e2 * 3 + c] = cb[e2][c];
                        }
                }
                __syncthreads();
            }
            const double *Dm = m == 0 ? DB : D;
            for (int j0 = 0; j0 < 9; j0 += ST_JCH) {
                double acc[ST_PER_T];
#pragma unroll
                for (int r = 0; r < ST_PER_T; r++) acc[r] = 0.0;
                for (int gp = 0; gp < 9; gp++) {
                    // test side: A2[(jn - j0)*10 + je][q] = WET sum_k psi_k(jn) D[gp][q][je][k]
                    const double w = base[gp].WET;
                    for (int it = t; it < ST_JCH * ST_NEQ * ST_NQ; it += ST_THREADS) {
                        const int row = it / ST_NQ, q = it % ST_NQ;
                        const int jn = j0 + row / ST_NEQ, je = row % ST_NEQ;
                        const double *dd = Dm + ((size_t)(gp * ST_NQ + q) * ST_NEQ + je) * 3;
                        A2[row * ST_A2 + q] = w * (s_bfn[gp][jn] * dd[0] + s_dFx[gp][jn] * dd[1]
                                                   + s_dFy[gp][jn] * dd[2]);
                    }
                    __syncthreads();
                    // trial side; chunk output c = ((jn - j0)*9 + inod)*100 + jeq*10 + ieq
#pragma unroll
                    for (int r = 0; r < ST_PER_T; r++) {
                        const int c = t + r * ST_THREADS;
                        if (c < ST_CH_OUT) {
                            const int ji = c / 100, rr = c % 100;
                            const int jl = ji / 9, in = ji % 9;
                            const int je = rr / 10, ie = rr % 10;
                            const double *a2 = A2 + (jl * ST_NEQ + je) * ST_A2;
                            const int q0 = st_q(ie, 0);
                            double v = a2[q0] * s_bfn[gp][in] + a2[q0 + 1] * s_dFx[gp][in]
                                       + a2[q0 + 2] * s_dFy[gp][in];
                            if (ie < 3) v = v + a2[q0 + 3] * s_lap[gp][in];
                            acc[r] = acc[r] + v;
                        }
                    }
                    __syncthreads();
                }
#pragma unroll
                for (int r = 0; r < ST_PER_T; r++) {
                    const int c = t + r * ST_THREADS;
                    if (c < ST_CH_OUT) out[(size_t)m * ST_BLK + j0 * 900 + c] = acc[r];
                }
            }
        }
    }
}

// one thread per AIJ entry of a node-pair block of the 10-unknown pattern
__global__ void k_stability_gather(const GatherArgs g, const int64_t *__restrict__ rowptr10,
                                   const int32_t *__restrict__ boff10, const double *__restrict__ es,
                                   int nk, const double *__restrict__ kw, double *const *A,
                                   double *B)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nblocks * 100) return;
    const int blk = (int)(t / 100), r = (int)(t % 100);
    const int jeq = r / 10, ieq = r % 10;
    const int64_t slot = rowptr10[(int64_t)g.brow[blk] * ST_NEQ + jeq] + boff10[blk] + ieq;
    double sb = 0.0, s0 = 0.0, sp = 0.0, sn = 0.0;
    for (int c = g.bptr[blk]; c < g.bptr[blk + 1]; c++) {
        const int64_t con = g.bcon[c];                    // e*81 + jnod*9 + inod
        const int64_t e = con / 81, ji = con % 81;
        const double *src = es + (size_t)e * 4 * ST_BLK + ji * 100 + r;
        sb = sb + src[0];
        s0 = s0 + src[ST_BLK];
        sp = sp + src[2 * ST_BLK];
        sn = sn + src[3 * ST_BLK];
    }
    if (B) B[slot] = B[slot] + sb;
    const double a1 = (sp - sn) * 0.5, a2 = (sp + sn) * 0.5 - s0;
    for (int k = 0; k < nk; k++) {   // A(K) = s0 + K (a1 + K a2), two FMAs per wavenumber
        const double K = kw[k];
        A[k][slot] = A[k][slot] + __fma_rn(K, __fma_rn(K, a2, a1), s0);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side

__global__ void k_boff10(int n, const int32_t *__restrict__ boff6, int32_t *__restrict__ boff10)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) boff10[i] = boff6[i] / 6 * 10;
}

cudaError_t stab_upload_tables(const GaussTables &t, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
#define UP(sym, src)                                                                       \
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(sym, src, sizeof(src), 0, cudaMemcpyHostToDevice, s);
    UP(s_w, t.w)
    UP(s_bfn, t.bfn)
    UP(s_dfdc, t.dfdc)
    UP(s_dfde, t.dfde)
    UP(s_d2c, t.d2fdc2)
    UP(s_d2e, t.d2fde2)
    UP(s_d2ce, t.d2fdce)
#undef UP
    return e;
}

}  // namespace vefem

using namespace vefem;

namespace {

int sfail(vefem_ctx *c, int code, const std::string &m)
{
    c->err = m;
    return code;
}

#define SCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t _e = (call);                                                           \
        if (_e != cudaSuccess)                                                             \
            return sfail(ctx, VEFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// The 10-unknown pattern from the frozen 6-unknown one: every node-pair block
// becomes a 10 x 10 block, the extra (arclength) columns and rows are dropped.
int stab_pattern(vefem_ctx *ctx)
{
    if (!ctx->h_rowptr10.empty()) return VEFEM_OK;
    const int64_t nn = ctx->nnodes;
    std::vector<int64_t> rp(nn * ST_NEQ + 1, 0);
    std::vector<int32_t> ci;
    for (int64_t n = 0; n < nn; n++) {
        const int64_t r0 = ctx->h_rowptr[n * 6], r1 = ctx->h_rowptr[n * 6 + 1];
        std::vector<int32_t> cols;
        for (int64_t s = r0; s < r1; s++) {
            const int32_t c = ctx->h_colind[s];
            if (c < nn * 6 && c % 6 == 0) cols.push_back(c / 6);
        }
        for (int q = 0; q < ST_NEQ; q++) {
            for (int32_t cn : cols)
                for (int f = 0; f < ST_NEQ; f++) ci.push_back(cn * ST_NEQ + f);
            rp[n * ST_NEQ + q + 1] = (int64_t)ci.size();
        }
    }
    ctx->h_rowptr10.swap(rp);
    ctx->h_colind10.swap(ci);
    SCK(cudaMalloc((void **)&ctx->d_rowptr10, ctx->h_rowptr10.size() * sizeof(int64_t)));
    SCK(cudaMemcpy(ctx->d_rowptr10, ctx->h_rowptr10.data(), ctx->h_rowptr10.size() * sizeof(int64_t),
                   cudaMemcpyHostToDevice));
    SCK(cudaMalloc((void **)&ctx->d_boff10, std::max(1, ctx->nblocks) * sizeof(int32_t)));
    if (ctx->nblocks > 0)
        k_boff10<<<(ctx->nblocks + 255) / 256, 256, 0, ctx->stream>>>(ctx->nblocks, ctx->d_boff, ctx->d_boff10);
    SCK(cudaGetLastError());
    SCK(cudaStreamSynchronize(ctx->stream));
    return VEFEM_OK;
}

}  // namespace

extern "C" int vefem_stability_pattern(vefem_ctx *ctx, int64_t *n, int64_t *nnz, int64_t *rowptr,
                                       int32_t *colind)
{
    if (!ctx || !n || !nnz) return VEFEM_ERR_ARG;
    SCK(cudaSetDevice(ctx->device));
    if (int rc = stab_pattern(ctx)) return rc;
    *n = (int64_t)ctx->h_rowptr10.size() - 1;
    *nnz = (int64_t)ctx->h_colind10.size();
    if (rowptr) std::copy(ctx->h_rowptr10.begin(), ctx->h_rowptr10.end(), rowptr);
    if (colind) std::copy(ctx->h_colind10.begin(), ctx->h_colind10.end(), colind);
    return VEFEM_OK;
}

extern "C" int vefem_stability_assemble(vefem_ctx *ctx, const double *TLb, int nk, const double *kw,
                                        int flags, double *const *A, double *B, int on_device)
{
    if (!ctx) return VEFEM_ERR_ARG;
    const int known = VEFEM_ZERO_FIRST | VEFEM_STAB_AS_WRITTEN;
    if (flags & ~known) return sfail(ctx, VEFEM_ERR_UNSUPPORTED, "unknown flag");
    if (!TLb || nk < 0 || (nk > 0 && (!kw || !A))) return sfail(ctx, VEFEM_ERR_ARG, "NULL argument");
    for (int k = 0; k < nk; k++)
        if (!A[k]) return sfail(ctx, VEFEM_ERR_ARG, "NULL A array");
    if (ctx->prm.form != FORM_T)
        return sfail(ctx, VEFEM_ERR_UNSUPPORTED, "stability assembly: T form only");
    SCK(cudaSetDevice(ctx->device));
    if (int rc = stab_pattern(ctx)) return rc;
    cudaStream_t s = ctx->stream;
    const int64_t N10 = (int64_t)ctx->nnodes * ST_NEQ, nnz10 = (int64_t)ctx->h_colind10.size();
    if (!ctx->d_ses) {
        SCK(cudaMalloc((void **)&ctx->d_ses, (size_t)ctx->nel * 4 * ST_BLK * sizeof(double)));
        SCK(cudaMalloc((void **)&ctx->d_tlb, (size_t)N10 * sizeof(double)));
        GaussTables gt;
        gauss_tables_host(&gt);
        SCK(stab_upload_tables(gt, s));
    }
    if (nk > ctx->stab_nk) {
        cudaFree(ctx->d_kw);
        cudaFree(ctx->d_Aptr);
        SCK(cudaMalloc((void **)&ctx->d_kw, nk * sizeof(double)));
        SCK(cudaMalloc((void **)&ctx->d_Aptr, nk * sizeof(double *)));
        ctx->stab_nk = nk;
    }
    // device pointers of the outputs (host buffers: staging arrays)
    std::vector<double *> dA(nk);
    double *dB = B;
    if (!on_device) {
        if (nk > ctx->stab_nk_stage) {
            cudaFree(ctx->d_Astage);
            SCK(cudaMalloc((void **)&ctx->d_Astage, (size_t)nk * nnz10 * sizeof(double)));
            ctx->stab_nk_stage = nk;
        }
        if (B && !ctx->d_Bstage) SCK(cudaMalloc((void **)&ctx->d_Bstage, (size_t)nnz10 * sizeof(double)));
        for (int k = 0; k < nk; k++) dA[k] = ctx->d_Astage + (size_t)k * nnz10;
        dB = B ? ctx->d_Bstage : nullptr;
        SCK(cudaMemcpyAsync(ctx->d_tlb, TLb, N10 * sizeof(double), cudaMemcpyHostToDevice, s));
        if (!(flags & VEFEM_ZERO_FIRST)) {
            for (int k = 0; k < nk; k++)
                SCK(cudaMemcpyAsync(dA[k], A[k], nnz10 * sizeof(double), cudaMemcpyHostToDevice, s));
            if (B) SCK(cudaMemcpyAsync(dB, B, nnz10 * sizeof(double), cudaMemcpyHostToDevice, s));
        }
    } else {
        for (int k = 0; k < nk; k++) dA[k] = A[k];
        SCK(cudaMemcpyAsync(ctx->d_tlb, TLb, N10 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    if (flags & VEFEM_ZERO_FIRST) {
        for (int k = 0; k < nk; k++) SCK(cudaMemsetAsync(dA[k], 0, nnz10 * sizeof(double), s));
        if (dB) SCK(cudaMemsetAsync(dB, 0, nnz10 * sizeof(double), s));
    }
    if (nk > 0) {
        SCK(cudaMemcpyAsync(ctx->d_kw, kw, nk * sizeof(double), on_device ? cudaMemcpyDeviceToDevice
                                                                          : cudaMemcpyHostToDevice, s));
        SCK(cudaMemcpyAsync(ctx->d_Aptr, dA.data(), nk * sizeof(double *), cudaMemcpyHostToDevice, s));
    }
    // element kernel
    StabArgs a;
    a.nel = ctx->nel;
    a.nnodes = ctx->nnodes;
    a.conn = ctx->d_conn;
    a.xy = ctx->d_xy;
    a.TLb = ctx->d_tlb;
    a.es = ctx->d_ses;
    a.kz = (flags & VEFEM_STAB_AS_WRITTEN) ? 0 : 1;
    const size_t smem = sizeof(double) * st_smem_doubles() + 9 * sizeof(StabBase);
    SCK(cudaFuncSetAttribute(k_stability, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    SCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_stability, ST_THREADS, smem));
    int sms = 0;
    SCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int grid = std::min<int>(ctx->nel, sms * std::max(1, occ));
    ctx->launches = 0;
    if (ctx->nel > 0) {
        k_stability<<<grid, ST_THREADS, smem, s>>>(a, ctx->prm);
        SCK(cudaGetLastError());
        ctx->launches++;
    }
    GatherArgs g;
    g.nnodes = ctx->nnodes;
    g.nblocks = ctx->nblocks;
    g.nex = 0;
    g.rowptr = ctx->d_rowptr;
    g.nptr = ctx->d_nptr;
    g.ncon = ctx->d_ncon;
    g.brow = ctx->d_brow;
    g.boff = ctx->d_boff;
    g.bptr = ctx->d_bptr;
    g.bcon = ctx->d_bcon;
    const int64_t nthr = (int64_t)ctx->nblocks * 100;
    if (nthr > 0) {
        k_stability_gather<<<(unsigned)((nthr + 255) / 256), 256, 0, s>>>(
            g, ctx->d_rowptr10, ctx->d_boff10, ctx->d_ses, nk, ctx->d_kw, ctx->d_Aptr, dB);
        SCK(cudaGetLastError());
        ctx->launches++;
    }
    if (!on_device) {
        for (int k = 0; k < nk; k++)
            SCK(cudaMemcpyAsync(A[k], dA[k], nnz10 * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (B) SCK(cudaMemcpyAsync(B, dB, nnz10 * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    SCK(cudaStreamSynchronize(s));
    return VEFEM_OK;
}
