/*
 * vefem_oracle.c -- CPU oracle for the element assembly of the viscoelastic
 * flow-around-a-cylinder solver (reference: AlexSp8/VE_flow_around_cylinder_Fortran).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product (the CUDA library) never links or calls it.
 *
 * It is a literal, scalar restatement of the reference Fortran, routine by
 * routine, with 3x3 tensors exactly as the Fortran declares them, and every
 * floating-point expression evaluated left to right in the order the Fortran
 * source writes it.  Build it with -ffp-contract=off (no FMA contraction) so
 * the arithmetic is plain IEEE binary64.
 *
 * Parity status: parity unpinned against the reference itself -- it cannot be
 * compiled on this machine or the GPU machine (Fortran + PETSc + MPI, no Fortran
 * compiler) and it ships no tests or golden vectors.  The restatement is
 * pinned instead by known-answer checks: homogeneous-flow patch tests against
 * the textbook constitutive equations (zero constitutive and continuity
 * residuals), a column-by-column replay of the FD Jacobian, FD against
 * central differences, and mirror symmetry.
 *
 * Index conventions: Fortran A(i,j) (1-based) is A[i-1][j-1] here.
 * Element unknowns TEMP_TL(inod,ieq) are tl[inod][ieq] (9 x 6), field order
 * Ux, Uy, P, Txx, Txy, Tyy (Tools_mod.F90:622-649).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Scalar type of the state-dependent arithmetic.  The default build is plain
 * binary64.  Built with -DORA_COMPLEX_STEP the same routines run on complex
 * numbers, and ora_cs_element_batch (end of file) differentiates residualBulk
 * by the complex step: column j of the element Jacobian is
 * Im(Res(x + i h e_j)) / h with h = 1e-30 (Squire & Trapp, SIAM Rev. 40, 1998;
 * Martins, Sturdza & Alonso, ACM TOMS 29, 2003).  No difference is taken, so
 * the column is exact to rounding: an oracle for the exact (linearised)
 * Jacobian, independent of the library's forward-mode dual numbers.  |x| is
 * continued as sign(Re x) x, the derivative of the absolute value away from 0. */
#ifdef ORA_COMPLEX_STEP
#include <complex.h>
typedef double _Complex real_t;
static inline real_t RABS(real_t z) { return creal(z) < 0.0 ? -z : z; }
#define RSQRT(z) csqrt(z)
#define REXP(z) cexp(z)
#else
typedef double real_t;
#define RABS(z) fabs(z)
#define RSQRT(z) sqrt(z)
#define REXP(z) exp(z)
#endif

#define NBF 9
#define NEQ 6
#define NGP 9
#define NEQ_F 2
#define NEQ_S 3
#define NDIM 2

enum { M_L_PTT = 0, M_M_L_PTT = 1, M_E_PTT = 2, M_M_E_PTT = 3,
       M_FENE_CR = 4, M_FENE_P = 5, M_GIESEKUS = 6 };
enum { FORM_T = 0, FORM_SQRT = 1 };

/* Run-time restatement of the compile-time parameters of Parameters_mod.F90
 * (Model_Name :101, Stress_Reform :122, ReN/WiN/BvN/VeN/DfN :98-111) and of
 * dt = huge(1d0) for steady runs (Physical_mod.F90:345). */
typedef struct {
    int model, form, nex;
    double ReN, WiN, BvN, VeN, DfN, Wi0, dt, eps;
} prm_t;

/* Gauss tables, Gauss_Quadrangle_mod.F90 layout (Nbf, Ngauss) -> [ig][inod] */
typedef struct {
    double w[NGP];
    double bfn[NGP][NBF], dfdc[NGP][NBF], dfde[NGP][NBF];
    double d2fdc2[NGP][NBF], d2fde2[NGP][NBF], d2fdce[NGP][NBF];
} gauss_t;

/* GaussPointQuantities, Global_Variables_mod.F90:56-84 (fields on this path) */
typedef struct {
    real_t GU[3][3], GUT[3][3], G_dot[3][3], GU_tr[3][3], GUT_tr[3][3], G_dot_tr[3][3];
    real_t P_tot[3][3], G2U[3][3];
    real_t U_f[3], dPdXi[3], dUfdt[3];
    real_t Momentum[3], Convection[3];
    real_t Continuity, P;
    real_t dTdXi[3][3][3], dCdXi[3][3][3], dSdXi[3][3][3];
    real_t S[3][3], dSdt[3][3];
    real_t Con_EQ[3][3], T_ve[3][3], C_Tensor[3][3];
    real_t f[3], g[2], dgdxi[2][3], f_T;
    double dXidci[3][3];
    double detJ, WET;
    real_t mag_con_EQ, tlsic, tlsme, tlsce, tdcs;
} gp_t;

/* NodeArrays, Global_Variables_mod.F90:86-110 (fields on this path) */
typedef struct {
    real_t tl[NBF][NEQ];
    real_t eu[2];
    double xi[NBF][3];                       /* geometry is never perturbed */
    double dFdXi[3][NBF], d2FdXi2[3][NBF];
    const double *bfn, *dfdc, *dfde, *d2fdc2, *d2fde2, *d2fdce;
} elem_t;

/* ---------------------------------------------------------------------- */
/* Gauss_Quadrangle_mod.F90                                                */

/* setQuadraticQuadrangle, Gauss_Quadrangle_mod.F90:405-478 */
static void quadratic_quadrangle(double c, double e, double *bfn, double *dfdc, double *dfde,
                                 double *d2fdc2, double *d2fde2, double *d2fdce)
{
    bfn[0] = +(1.0 - c) * c * (1.0 - e) * e / 4.0;
    bfn[1] = -(1.0 + c) * c * (1.0 - e) * e / 4.0;
    bfn[2] = +(1.0 + c) * c * (1.0 + e) * e / 4.0;
    bfn[3] = -(1.0 - c) * c * (1.0 + e) * e / 4.0;
    bfn[4] = -(1.0 + c) * (1.0 - c) * (1.0 - e) * e / 2.0;
    bfn[5] = +(1.0 + c) * c * (1.0 + e) * (1.0 - e) / 2.0;
    bfn[6] = +(1.0 + c) * (1.0 - c) * (1.0 + e) * e / 2.0;
    bfn[7] = -(1.0 - c) * c * (1.0 + e) * (1.0 - e) / 2.0;
    bfn[8] = +(1.0 + c) * (1.0 - c) * (1.0 + e) * (1.0 - e);

    dfdc[0] = +(1.0 - 2.0 * c) * (1.0 - e) * e / 4.0;
    dfdc[1] = -(1.0 + 2.0 * c) * (1.0 - e) * e / 4.0;
    dfdc[2] = +(1.0 + 2.0 * c) * (1.0 + e) * e / 4.0;
    dfdc[3] = -(1.0 - 2.0 * c) * (1.0 + e) * e / 4.0;
    dfdc[4] = -(-2.0 * c) * (1.0 - e) * e / 2.0;
    dfdc[5] = +(1.0 + 2.0 * c) * (1.0 + e) * (1.0 - e) / 2.0;
    dfdc[6] = +(-2.0 * c) * (1.0 + e) * e / 2.0;
    dfdc[7] = -(1.0 - 2.0 * c) * (1.0 + e) * (1.0 - e) / 2.0;
    dfdc[8] = +(-2.0 * c) * (1.0 + e) * (1.0 - e);

    d2fdc2[0] = +(-2.0) * (1.0 - e) * e / 4.0;
    d2fdc2[1] = -(+2.0) * (1.0 - e) * e / 4.0;
    d2fdc2[2] = +(+2.0) * (1.0 + e) * e / 4.0;
    d2fdc2[3] = -(-2.0) * (1.0 + e) * e / 4.0;
    d2fdc2[4] = -(-2.0) * (1.0 - e) * e / 2.0;
    d2fdc2[5] = +(+2.0) * (1.0 + e) * (1.0 - e) / 2.0;
    d2fdc2[6] = +(-2.0) * (1.0 + e) * e / 2.0;
    d2fdc2[7] = -(-2.0) * (1.0 + e) * (1.0 - e) / 2.0;
    d2fdc2[8] = +(-2.0) * (1.0 + e) * (1.0 - e);

    d2fdce[0] = +(1.0 - 2.0 * c) * (1.0 - 2.0 * e) / 4.0;
    d2fdce[1] = -(1.0 + 2.0 * c) * (1.0 - 2.0 * e) / 4.0;
    d2fdce[2] = +(1.0 + 2.0 * c) * (1.0 + 2.0 * e) / 4.0;
    d2fdce[3] = -(1.0 - 2.0 * c) * (1.0 + 2.0 * e) / 4.0;
    d2fdce[4] = -(-2.0 * c) * (1.0 - 2.0 * e) / 2.0;
    d2fdce[5] = +(1.0 + 2.0 * c) * (-2.0 * e) / 2.0;
    d2fdce[6] = +(-2.0 * c) * (1.0 + 2.0 * e) / 2.0;
    d2fdce[7] = -(1.0 - 2.0 * c) * (-2.0 * e) / 2.0;
    d2fdce[8] = +(-2.0 * c) * (-2.0 * e);

    dfde[0] = +(1.0 - c) * c * (1.0 - 2.0 * e) / 4.0;
    dfde[1] = -(1.0 + c) * c * (1.0 - 2.0 * e) / 4.0;
    dfde[2] = +(1.0 + c) * c * (1.0 + 2.0 * e) / 4.0;
    dfde[3] = -(1.0 - c) * c * (1.0 + 2.0 * e) / 4.0;
    dfde[4] = -(1.0 + c) * (1.0 - c) * (1.0 - 2.0 * e) / 2.0;
    dfde[5] = +(1.0 + c) * c * (-2.0 * e) / 2.0;
    dfde[6] = +(1.0 + c) * (1.0 - c) * (1.0 + 2.0 * e) / 2.0;
    dfde[7] = -(1.0 - c) * c * (-2.0 * e) / 2.0;
    dfde[8] = +(1.0 + c) * (1.0 - c) * (-2.0 * e);

    d2fde2[0] = +(1.0 - c) * c * (-2.0) / 4.0;
    d2fde2[1] = -(1.0 + c) * c * (-2.0) / 4.0;
    d2fde2[2] = +(1.0 + c) * c * (+2.0) / 4.0;
    d2fde2[3] = -(1.0 - c) * c * (+2.0) / 4.0;
    d2fde2[4] = -(1.0 + c) * (1.0 - c) * (-2.0) / 2.0;
    d2fde2[5] = +(1.0 + c) * c * (-2.0) / 2.0;
    d2fde2[6] = +(1.0 + c) * (1.0 - c) * (+2.0) / 2.0;
    d2fde2[7] = -(1.0 - c) * c * (-2.0) / 2.0;
    d2fde2[8] = +(1.0 + c) * (1.0 - c) * (-2.0);
}

/* setGaussPointsQuadrangle1D :54-78 (3-point rule with the 0+1d-8 "centre"),
 * setGaussPointsQuadrangle2D :82-101 (i outer = xi, j inner = eta),
 * setGaussWeightsQuadrangle1D/2D :152-200, bulk tables :318-374 */
static void gauss_tables(gauss_t *G)
{
    double p1[3], w1[3];
    p1[0] = 0.0 + 1.0e-8;
    p1[1] = +sqrt(3.0 / 5.0);
    p1[2] = -sqrt(3.0 / 5.0);
    w1[0] = 8.0 / 9.0;
    w1[1] = 5.0 / 9.0;
    w1[2] = 5.0 / 9.0;
    int ng = 0;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            G->w[ng] = w1[i] * w1[j];
            quadratic_quadrangle(p1[i], p1[j], G->bfn[ng], G->dfdc[ng], G->dfde[ng],
                                 G->d2fdc2[ng], G->d2fde2[ng], G->d2fdce[ng]);
            ng++;
        }
    }
}

/* 1-D edge tables for edge ied (1..4), setGaussBasisFunctionsQuadrangleEdge :243-314 */
static void gauss_edge_tables(int ied, double w[3], double bfn[3][NBF], double dfdc[3][NBF],
                              double dfde[3][NBF], double d2c[3][NBF], double d2e[3][NBF],
                              double d2ce[3][NBF])
{
    double p1[3], w1[3];
    p1[0] = 0.0 + 1.0e-8;
    p1[1] = +sqrt(3.0 / 5.0);
    p1[2] = -sqrt(3.0 / 5.0);
    w1[0] = 8.0 / 9.0;
    w1[1] = 5.0 / 9.0;
    w1[2] = 5.0 / 9.0;
    for (int ig = 0; ig < 3; ig++) {
        double c = 0, e = 0;
        switch (ied) {
        case 1: c = p1[ig]; e = -1.0; break;
        case 2: c = +1.0; e = p1[ig]; break;
        case 3: c = p1[ig]; e = +1.0; break;
        default: c = -1.0; e = p1[ig]; break;
        }
        w[ig] = w1[ig];
        quadratic_quadrangle(c, e, bfn[ig], dfdc[ig], dfde[ig], d2c[ig], d2e[ig], d2ce[ig]);
    }
}

/* ---------------------------------------------------------------------- */
/* Tools_mod.F90                                                           */

/* traceTensorReal :206-220 */
static real_t trace3(const real_t A[3][3])
{
    real_t t = 0.0;
    for (int i = 0; i < 3; i++) t = t + A[i][i];
    return t;
}

/* doubleDotProductReal :262-278 -- A:B^T, i outer, j inner */
static real_t ddot3(const real_t A[3][3], const real_t B[3][3])
{
    real_t s = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) s = s + A[i][j] * B[j][i];
    return s;
}

/* Fortran matmul for 3x3: C(i,j) = sum_k A(i,k) B(k,j), k ascending from zero */
static void matmul3(const real_t A[3][3], const real_t B[3][3], real_t C[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            real_t s = 0.0;
            for (int k = 0; k < 3; k++) s = s + A[i][k] * B[k][j];
            C[i][j] = s;
        }
}

/* dot_product over the 9 element nodes */
static real_t dot9(const real_t *a, int sa, const double *b)
{
    real_t s = 0.0;
    for (int n = 0; n < NBF; n++) s = s + a[n * sa] * b[n];
    return s;
}

static real_t dot3(const real_t *a, const real_t *b)
{
    real_t s = 0.0;
    for (int n = 0; n < 3; n++) s = s + a[n] * b[n];
    return s;
}

/* getStressComponent :769-793 (order 11, 12, 22, 13, 23, 33) */
static void stress_component(int i, int istart, int *j, int *k)
{
    static const int J[6] = {0, 0, 1, 0, 1, 2}, K[6] = {0, 1, 1, 2, 2, 2};
    *j = J[i - istart];
    *k = K[i - istart];
}

/* inverseTensor2D :129-146 with determinant2D :78-87 */
static void inverse2(const real_t A[2][2], real_t AI[2][2])
{
    real_t detA = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    AI[0][0] = A[1][1];
    AI[0][1] = -A[0][1];
    AI[1][0] = -A[1][0];
    AI[1][1] = A[0][0];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) AI[i][j] = AI[i][j] / detA;
}

/* ---------------------------------------------------------------------- */
/* Element_Calculations_mod.F90                                            */

static const double I3[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

/* setElementBasisFunctions :222-243 */
static void set_element_basis(const gauss_t *G, int ig, elem_t *E)
{
    E->bfn = G->bfn[ig];
    E->dfdc = G->dfdc[ig];
    E->dfde = G->dfde[ig];
    E->d2fdc2 = G->d2fdc2[ig];
    E->d2fde2 = G->d2fde2[ig];
    E->d2fdce = G->d2fdce[ig];
}

/* basis2D :308-361, idir = [1, 2] (Physical_mod.F90:98) */
static void basis2d(elem_t *E, gp_t *g)
{
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) g->dXidci[a][b] = 0.0;
    for (int inod = 0; inod < NBF; inod++) {
        for (int j = 0; j < 3; j++) {
            g->dXidci[0][j] = g->dXidci[0][j] + E->dfdc[inod] * E->xi[inod][j];
            g->dXidci[1][j] = g->dXidci[1][j] + E->dfde[inod] * E->xi[inod][j];
        }
    }
    double dxdc = g->dXidci[0][0], dydc = g->dXidci[0][1];
    double dxde = g->dXidci[1][0], dyde = g->dXidci[1][1];
    g->detJ = dxdc * dyde - dxde * dydc;
    double dcdx = dyde / g->detJ;
    double dedx = -dydc / g->detJ;
    double dcdy = -dxde / g->detJ;
    double dedy = dxdc / g->detJ;
    for (int a = 0; a < 3; a++)
        for (int n = 0; n < NBF; n++) {
            E->dFdXi[a][n] = 0.0;
            E->d2FdXi2[a][n] = 0.0;
        }
    for (int n = 0; n < NBF; n++) {
        E->dFdXi[0][n] = (dcdx * E->dfdc[n] + dedx * E->dfde[n]);
        E->dFdXi[1][n] = (dcdy * E->dfdc[n] + dedy * E->dfde[n]);
        E->d2FdXi2[0][n] = (dcdx * dcdx) * E->d2fdc2[n] + (dedx * dedx) * E->d2fde2[n]
                           + 2.0 * dcdx * dedx * E->d2fdce[n];
        E->d2FdXi2[1][n] = (dcdy * dcdy) * E->d2fdc2[n] + (dedy * dedy) * E->d2fde2[n]
                           + 2.0 * dcdy * dedy * E->d2fdce[n];
    }
}

/* setFlowUnknowns :449-533 (Problem%name = 'Cylinder_2D', no projection) */
static void set_flow_unknowns(const elem_t *E, gp_t *g)
{
    for (int i = 0; i < 3; i++) {
        g->U_f[i] = 0.0;
        g->dPdXi[i] = 0.0;
        for (int j = 0; j < 3; j++) {
            g->GU[i][j] = 0.0;
            g->G2U[i][j] = 0.0;
        }
    }
    g->P = 0.0;
    for (int i = 0; i < NEQ_F; i++) {
        g->U_f[i] = dot9(&E->tl[0][i], NEQ, E->bfn);
        for (int j = 0; j < 3; j++) {
            g->GU[j][i] = dot9(&E->tl[0][i], NEQ, E->dFdXi[j]);
            g->G2U[j][i] = dot9(&E->tl[0][i], NEQ, E->d2FdXi2[j]);
        }
        g->dPdXi[i] = dot9(&E->tl[0][NEQ_F], NEQ, E->dFdXi[i]);
    }
    g->P = dot9(&E->tl[0][NEQ_F], NEQ, E->bfn);

    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            g->S[a][b] = 0.0;
            for (int c = 0; c < 3; c++) g->dSdXi[a][b][c] = 0.0;
        }
    int istart = NEQ - NEQ_S;
    for (int i = istart; i < NEQ; i++) {
        int j, k;
        stress_component(i, istart, &j, &k);
        g->S[j][k] = dot9(&E->tl[0][i], NEQ, E->bfn);
        g->S[k][j] = g->S[j][k];
        for (int idim = 0; idim < 3; idim++)
            g->dSdXi[j][k][idim] = dot9(&E->tl[0][i], NEQ, E->dFdXi[idim]);
        for (int idim = 0; idim < 3; idim++) g->dSdXi[k][j][idim] = g->dSdXi[j][k][idim];
    }
}

/* setFlowKinematics :605-634 with N = Ndim = 2 */
static void set_flow_kinematics(gp_t *g)
{
    const int N = NDIM;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GUT[i][j] = g->GU[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->G_dot[i][j] = g->GU[i][j] + g->GUT[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GU_tr[i][j] = g->GU[i][j];
    real_t tr = trace3(g->GU);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) g->GU_tr[i][j] = g->GU[i][j] - tr * I3[i][j] / (real_t)N;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GUT_tr[i][j] = g->GU_tr[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->G_dot_tr[i][j] = g->GU_tr[i][j] + g->GUT_tr[i][j];
}

/* ---------------------------------------------------------------------- */
/* Constitutive_Models_mod.F90 (T form)                                    */

/* setFENEMaterialDerivative :272-311, steady (no Transient term) */
static real_t fene_material_derivative(const prm_t *p, real_t WiN, const gp_t *g)
{
    real_t dfdXi[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) dfdXi[c] = dfdXi[c] + g->dTdXi[i][i][c];
    if (p->model == M_FENE_P) {
        for (int c = 0; c < 3; c++) dfdXi[c] = (WiN / (1.0 - p->BvN)) * dfdXi[c] / p->VeN;
    } else {
        for (int c = 0; c < 3; c++)
            dfdXi[c] = (WiN / (1.0 - p->BvN)) * dfdXi[c] / (p->VeN - (real_t)NDIM);
    }
    real_t MDfDt = 0.0;
    for (int i = 0; i < 3; i++) MDfDt = MDfDt + g->U_f[i] * dfdXi[i];
    return MDfDt;
}

/* conEQ_* :96-268 */
static void con_eq_T(const prm_t *p, real_t WiN, gp_t *g)
{
    real_t trT = trace3(g->S);
    double BvN = p->BvN, VeN = p->VeN;
    switch (p->model) {
    case M_L_PTT:
        g->f_T = 1.0 + (VeN * WiN * trT) / (1.0 - BvN);
        g->f[0] = 1.0; g->f[1] = g->f_T; g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_M_L_PTT:
        g->f_T = 1.0 + (VeN * WiN * trT) / (1.0 - BvN);
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->g[0];
        break;
    case M_E_PTT:
        g->f_T = REXP(VeN * WiN * trT / (1.0 - BvN));
        g->f[0] = 1.0; g->f[1] = g->f_T; g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_M_E_PTT:
        g->f_T = REXP(VeN * WiN * trT / (1.0 - BvN));
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->g[0];
        break;
    case M_GIESEKUS:
        g->f_T = VeN * WiN / (1.0 - BvN);
        g->f[0] = 1.0; g->f[1] = 1.0; g->f[2] = g->f_T;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_FENE_CR: {
        g->f_T = 1.0 + ((WiN * trT / (1.0 - BvN))) / (VeN - (real_t)NDIM);
        g->f[0] = g->f_T;
        real_t MDfDt = fene_material_derivative(p, WiN, g);
        g->f[1] = g->f_T - (WiN * MDfDt / g->f_T);
        g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->g[0];
        break;
    }
    default: { /* M_FENE_P */
        g->f_T = 1.0 + (WiN * trT / (1.0 - BvN)) / VeN;
        g->f[0] = 1.0;
        real_t MDfDt = fene_material_derivative(p, WiN, g);
        g->f[1] = g->f_T - (WiN * MDfDt / g->f_T);
        g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = g->f_T;
        break;
    }
    }
}

/* setStressTensor :335-349 */
static void set_stress_tensor_T(const prm_t *p, real_t WiN, gp_t *g)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            g->P_tot[i][j] = g->T_ve[i][j] + p->BvN * g->G_dot_tr[i][j] - g->P * I3[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            g->C_Tensor[i][j] = WiN * (g->T_ve[i][j] / (1.0 - p->BvN)) + g->g[0] * I3[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->C_Tensor[i][j] = (1.0 / g->g[1]) * g->C_Tensor[i][j];
}

/* strongFormConEQ :55-92 with setUpperConvectedDerivativeT :315-331 */
static void strong_form_con_eq_T(const prm_t *p, real_t WiN, gp_t *g)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            g->T_ve[i][j] = g->S[i][j];
            for (int k = 0; k < 3; k++) g->dTdXi[i][j][k] = g->dSdXi[i][j][k];
        }
    con_eq_T(p, WiN, g);
    set_stress_tensor_T(p, WiN, g);

    real_t UCD[3][3], M1[3][3], M2[3][3], Tve2[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = g->dSdt[i][j];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] + g->U_f[k] * g->dSdXi[i][j][k];
    matmul3(g->GUT_tr, g->S, M1);
    matmul3(g->S, g->GU_tr, M2);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] - M1[i][j] - M2[i][j];
    matmul3(g->S, g->S, Tve2);

    real_t term_I = 0.0;
    if (p->model == M_FENE_P) {
        real_t MDfDt = fene_material_derivative(p, WiN, g);
        term_I = MDfDt / (g->f_T);
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            real_t c = WiN * UCD[i][j] + (g->f[2]) * Tve2[i][j];
            c = c + (g->f[1]) * g->S[i][j];
            c = c - g->f[0] * (1.0 - p->BvN) * (g->G_dot_tr[i][j] + term_I * I3[i][j]);
            g->Con_EQ[i][j] = c;
        }
}

/* ---------------------------------------------------------------------- */
/* Constitutive_Models_SQRT_mod.F90                                        */

/* WTensor2D :513-530 with omegaNominator2DReal :534-543, omegaDenominator2DReal :575-584 */
static void wtensor2d(const real_t S[2][2], const real_t GUT[2][2], real_t W[2][2])
{
    real_t n = -S[0][0] * GUT[1][0] + S[0][1] * (GUT[0][0] - GUT[1][1]) + S[1][1] * GUT[0][1];
    real_t d = S[0][0] + S[1][1];
    W[0][0] = 0.0;
    W[1][1] = 0.0;
    W[0][1] = n / d;
    W[1][0] = -W[0][1];
}

/* setOmegaTensor :420-455 */
static void omega_tensor(const real_t S3[3][3], const real_t GUT3[3][3], real_t W[3][3])
{
    real_t s[2][2], gt[2][2], w[2][2];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            s[i][j] = S3[i][j];
            gt[i][j] = GUT3[i][j];
        }
    wtensor2d(s, gt, w);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) W[i][j] = 0.0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) W[i][j] = w[i][j];
}

/* conEQ_*_SQRT :153-375 */
static void con_eq_sqrt(const prm_t *p, gp_t *g)
{
    const real_t N = (real_t)NDIM;
    double VeN = p->VeN;
    real_t trC = trace3(g->C_Tensor);
    for (int a = 0; a < 2; a++)
        for (int c = 0; c < 3; c++) g->dgdxi[a][c] = 0.0;
    switch (p->model) {
    case M_L_PTT:
        g->f_T = 1.0 + VeN * (trC - N);
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_M_L_PTT:
        g->f_T = 1.0 + VeN * (trC - N);
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->f_T;
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) g->dgdxi[0][c] = g->dgdxi[0][c] + g->dCdXi[i][i][c];
        for (int c = 0; c < 3; c++) g->dgdxi[0][c] = VeN * (g->dgdxi[0][c]);
        for (int c = 0; c < 3; c++) g->dgdxi[1][c] = g->dgdxi[0][c];
        break;
    case M_E_PTT:
        g->f_T = REXP(VeN * (trC - N));
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_M_E_PTT:
        g->f_T = REXP(VeN * (trC - N));
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->f_T;
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) g->dgdxi[0][c] = g->dgdxi[0][c] + g->dCdXi[i][i][c];
        for (int c = 0; c < 3; c++) g->dgdxi[0][c] = VeN * (g->f_T) * (g->dgdxi[0][c]);
        for (int c = 0; c < 3; c++) g->dgdxi[1][c] = g->dgdxi[0][c];
        break;
    case M_GIESEKUS:
        g->f_T = 1.0 - 2.0 * VeN;
        g->f[0] = 1.0 - VeN; g->f[1] = 1.0 - 2.0 * VeN; g->f[2] = VeN;
        g->g[0] = 1.0; g->g[1] = 1.0;
        break;
    case M_FENE_CR:
        g->f_T = (VeN - N) / (VeN - trC);
        g->f[0] = g->f_T; g->f[1] = g->f[0]; g->f[2] = 0.0;
        g->g[0] = g->f_T; g->g[1] = g->f_T;
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) g->dgdxi[0][c] = g->dgdxi[0][c] + g->dCdXi[i][i][c];
        for (int c = 0; c < 3; c++) g->dgdxi[0][c] = (g->f_T) * (g->dgdxi[0][c]) / (VeN - trC);
        for (int c = 0; c < 3; c++) g->dgdxi[1][c] = g->dgdxi[0][c];
        break;
    default: /* M_FENE_P */
        g->f_T = (VeN - N) / (VeN - trC);
        g->f[0] = 1.0; g->f[1] = g->f_T; g->f[2] = 0.0;
        g->g[0] = 1.0; g->g[1] = g->f_T;
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) g->dgdxi[1][c] = g->dgdxi[1][c] + g->dCdXi[i][i][c];
        for (int c = 0; c < 3; c++) g->dgdxi[1][c] = (g->f_T) * (g->dgdxi[1][c]) / (VeN - trC);
        break;
    }
}

/* setCTensorSQRT :379-393 */
static void set_c_tensor_sqrt(gp_t *g)
{
    matmul3(g->S, g->S, g->C_Tensor);
    for (int k = 0; k < 3; k++) {
        real_t dS[3][3], A[3][3], B[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) dS[i][j] = g->dSdXi[i][j][k];
        matmul3(dS, g->S, A);
        matmul3(g->S, dS, B);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) g->dCdXi[i][j][k] = A[i][j] + B[i][j];
    }
}

/* setStressTensorSQRT :483-509 */
static void set_stress_tensor_sqrt(const prm_t *p, real_t WiN, gp_t *g)
{
    double BvN = p->BvN;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            g->T_ve[i][j] = (g->g[1]) * (g->C_Tensor[i][j]) - (g->g[0]) * I3[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->T_ve[i][j] = ((1.0 - BvN) / WiN) * (g->T_ve[i][j]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            g->P_tot[i][j] = g->T_ve[i][j] + BvN * (g->G_dot_tr[i][j]) - (g->P) * I3[i][j];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                g->dTdXi[i][j][k] = (g->dgdxi[1][k]) * (g->C_Tensor[i][j])
                                    + (g->g[1]) * (g->dCdXi[i][j][k])
                                    - (g->dgdxi[0][k]) * I3[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                g->dTdXi[i][j][k] = ((1.0 - BvN) / WiN) * (g->dTdXi[i][j][k]);
}

/* strongFormConEQ_SQRT :120-149, setUpperConvectedDerivativeSQRT :397-416,
 * setSInverse :459-479 */
static void strong_form_con_eq_sqrt(const prm_t *p, real_t WiN, gp_t *g)
{
    set_c_tensor_sqrt(g);
    con_eq_sqrt(p, g);
    set_stress_tensor_sqrt(p, WiN, g);

    real_t UCD[3][3], W[3][3], M1[3][3], M2[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = g->dSdt[i][j];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                UCD[i][j] = UCD[i][j] + (g->U_f[k]) * (g->dSdXi[i][j][k]);
    omega_tensor(g->S, g->GUT_tr, W);
    matmul3(g->S, g->GU_tr, M1);
    matmul3(W, g->S, M2);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] - M1[i][j] - M2[i][j];

    real_t s2[2][2], si2[2][2], SI[3][3], SS[3][3], S3[3][3];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) s2[i][j] = g->S[i][j];
    inverse2(s2, si2);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) SI[i][j] = 0.0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) SI[i][j] = si2[i][j];
    matmul3(g->S, g->S, SS);
    matmul3(g->S, SS, S3);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            real_t term = (g->f[2]) * S3[i][j] + (g->f[1]) * g->S[i][j] - (g->f[0]) * SI[i][j];
            g->Con_EQ[i][j] = WiN * UCD[i][j] + term / 2.0;
        }
}

/* strongFormMomentum :658-683 */
static void strong_form_momentum(const prm_t *p, gp_t *g)
{
    real_t div_Tve[3] = {0.0, 0.0, 0.0}, div_Ptot[3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) div_Tve[i] = div_Tve[i] + g->dTdXi[j][i][j];
    for (int i = 0; i < 3; i++)
        div_Ptot[i] = -g->dPdXi[i] + div_Tve[i]
                      + p->BvN * (g->G2U[0][i] + g->G2U[1][i] + g->G2U[2][i]);
    for (int i = 0; i < 3; i++) {
        real_t s = 0.0;
        for (int k = 0; k < 3; k++) s = s + g->U_f[k] * g->GU[k][i];
        g->Convection[i] = g->dUfdt[i] + s;
    }
    for (int i = 0; i < 3; i++) g->Momentum[i] = p->ReN * (g->Convection[i]) - div_Ptot[i];
}

/* setContinuationParameter :577-601, strongFormEquations :537-573 */
static real_t strong_form_equations(const prm_t *p, const elem_t *E, gp_t *g)
{
    real_t WiN = p->WiN;
    if (p->nex > 0) WiN = p->Wi0 * E->eu[p->nex - 1];
    set_flow_kinematics(g);
    for (int i = 0; i < 3; i++) {
        g->dUfdt[i] = 0.0;
        for (int j = 0; j < 3; j++) g->dSdt[i][j] = 0.0;
    }
    if (p->form == FORM_SQRT)
        strong_form_con_eq_sqrt(p, WiN, g);
    else
        strong_form_con_eq_T(p, WiN, g);
    strong_form_momentum(p, g);
    g->Continuity = trace3(g->GU); /* strongFormContinuity :687-697 */
    return WiN;
}

/* setStabilizationTerms :701-773 */
static void set_stabilization_terms(const prm_t *p, real_t WiN, const elem_t *E, gp_t *g)
{
    double BvN = p->BvN, ReN = p->ReN, DfN = p->DfN, dt = p->dt;
    real_t Helem = 0.0, tsugn = 0.0;
    for (int n = 0; n < NBF; n++) {
        Helem = Helem + E->dFdXi[0][n] * E->dFdXi[0][n] + E->dFdXi[1][n] * E->dFdXi[1][n]
                + E->dFdXi[2][n] * E->dFdXi[2][n];
        real_t dF[3] = {E->dFdXi[0][n], E->dFdXi[1][n], E->dFdXi[2][n]};
        tsugn = tsugn + RABS(dot3(g->U_f, dF));
    }
    Helem = 1.0 / RSQRT(Helem);

    real_t double_dot_T = ddot3(g->T_ve, g->T_ve);
    real_t double_dot_G = ddot3(g->G_dot_tr, g->G_dot_tr);
    real_t Ha = RSQRT(((1.0 - BvN) / WiN) * ((1.0 - BvN) / WiN) + 0.5 * double_dot_T);
    Ha = Ha / RSQRT(1.0 + 0.5 * double_dot_G);

    real_t H2 = Helem * Helem;
    real_t t1 = ReN / dt, t2 = ReN * tsugn, t3 = BvN / H2, t4 = Ha / H2;
    g->tlsme = t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4;
    g->tlsme = 1.0 / RSQRT(g->tlsme);
    g->tlsic = H2 / (g->tlsme);

    real_t double_dot_S = ddot3(g->S, g->S), double_dot_C;
    g->tdcs = 0.5 * double_dot_S;
    if (p->form == FORM_SQRT) {
        double_dot_C = ddot3(g->C_Tensor, g->C_Tensor);
    } else {
        g->tdcs = (g->tdcs) + ((1.0 - BvN) / WiN) * ((1.0 - BvN) / WiN);
        double_dot_C = double_dot_T;
    }
    g->tdcs = H2 / RSQRT(g->tdcs);
    if (DfN > 1.0e-12) g->tdcs = 0.0;

    g->mag_con_EQ = ddot3(g->Con_EQ, g->Con_EQ);
    g->mag_con_EQ = RSQRT(0.5 * g->mag_con_EQ);

    real_t s1 = WiN / dt, s2 = WiN * tsugn, s3 = WiN * RSQRT(0.5 * double_dot_G), s4 = g->f[1];
    real_t s5 = g->f[2] * RSQRT(0.5 * double_dot_C), s6 = (g->tdcs) * (g->mag_con_EQ) / H2;
    real_t s7 = DfN / H2;
    g->tlsce = s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4 + s5 * s5 + s6 * s6 + s7 * s7;
    g->tlsce = 1.0 / RSQRT(g->tlsce);
}

/* ---------------------------------------------------------------------- */
/* Residuals_mod.F90                                                       */

/* momentumMain :44-86 (T) and momentumMainSQRT :295-337 with LSCEMomentumSQRT :388-433 */
static void momentum_main(const prm_t *p, real_t WiN, const elem_t *E, int inod, const gp_t *g,
                          real_t *res)
{
    double bifn = E->bfn[inod];
    real_t dF[3] = {E->dFdXi[0][inod], E->dFdXi[1][inod], E->dFdXi[2][inod]};
    for (int i = 0; i < NEQ_F; i++) {
        real_t lsme_term = (g->tlsme) * p->ReN * dot3(g->U_f, dF);  /* LSMEMomentum :161-173 */
        lsme_term = lsme_term * (g->Momentum[i]);
        real_t lsic_term = g->tlsic * dF[i];                        /* LSICMomentum :177-187 */
        lsic_term = lsic_term * (g->Continuity);
        real_t lsce[3][3];
        if (p->form == FORM_SQRT) {
            real_t GUT_lsce[3][3], GU_lsce[3][3], W_lsce[3][3], M1[3][3], M2[3][3];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) GUT_lsce[a][b] = 0.0;
            for (int b = 0; b < 3; b++) GUT_lsce[i][b] = dF[b];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) GU_lsce[a][b] = GUT_lsce[b][a];
            omega_tensor(g->S, GUT_lsce, W_lsce);
            matmul3(g->S, GU_lsce, M1);
            matmul3(W_lsce, g->S, M2);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    real_t ucd = -M1[a][b] - M2[a][b];
                    lsce[a][b] = (g->tlsce) * ucd * (1.0 - p->BvN) / WiN;
                }
        } else {                                                    /* LSCEMomentumT :191-219 */
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) lsce[a][b] = -g->tlsce * (a == i ? dF[b] : 0.0);
        }
        real_t lsce_term = ddot3(lsce, g->Con_EQ);
        real_t Pi[3] = {g->P_tot[i][0], g->P_tot[i][1], g->P_tot[i][2]};
        res[i] = p->ReN * (g->Convection[i]) * bifn + dot3(Pi, dF) + lsme_term + lsic_term
                 + lsce_term;
    }
}

/* continuityBulkMain :90-110 with LSMEContinuity :223-234 */
static void continuity_main(const elem_t *E, int inod, const gp_t *g, real_t *res)
{
    double bifn = E->bfn[inod];
    real_t dF[3] = {E->dFdXi[0][inod], E->dFdXi[1][inod], E->dFdXi[2][inod]};
    real_t lsme_term = g->tlsme * dot3(dF, g->Momentum);
    res[NEQ_F] = (g->Continuity) * bifn + lsme_term;
}

/* stressesBulkMain :114-157 (T) and stressesBulkMainSQRT :341-384 */
static void stresses_main(const prm_t *p, real_t WiN, const elem_t *E, int inod, const gp_t *g,
                          real_t *res)
{
    double bifn = E->bfn[inod];
    real_t dF[3] = {E->dFdXi[0][inod], E->dFdXi[1][inod], E->dFdXi[2][inod]};
    int istart = NEQ - NEQ_S;
    for (int i = istart; i < NEQ; i++) {
        int j, k;
        stress_component(i, istart, &j, &k);
        /* LSMEStressT :238-256 / LSMEStressSQRT :437-455 */
        real_t lsme_term = -dF[k] * g->Momentum[j];
        if (j != k) lsme_term = lsme_term - dF[j] * g->Momentum[k];
        if (p->form == FORM_SQRT)
            lsme_term = (g->tlsme) * lsme_term * WiN;
        else
            lsme_term = g->tlsme * lsme_term * (1.0 - p->BvN);
        /* LSCEStressT :260-276 / LSCEStressSQRT :459-475 */
        real_t lsce_term = WiN * dot3(g->U_f, dF);
        if (p->form == FORM_SQRT) lsce_term = lsce_term + (g->f_T) * bifn / 2.0;
        lsce_term = (g->tlsce) * lsce_term;
        lsce_term = lsce_term * (g->Con_EQ[j][k]);
        /* DCSStressT :280-291 / DCSStressSQRT :479-490 */
        const real_t *grad = (p->form == FORM_SQRT) ? g->dSdXi[j][k] : g->dTdXi[j][k];
        real_t dcs_term = (g->tdcs) * dot3(grad, dF);
        dcs_term = dcs_term * (g->mag_con_EQ);
        res[i] = (g->Con_EQ[j][k]) * bifn + p->DfN * dot3(grad, dF) + lsme_term + lsce_term
                 + dcs_term;
    }
}

/* ---------------------------------------------------------------------- */
/* Equations_mod.F90                                                       */

/* residualBulk :59-98 with equationsResidualsBulkMain :102-144 */
static void residual_bulk(const prm_t *p, const gauss_t *G, elem_t *E, real_t Res[NBF][NEQ])
{
    gp_t g;
    memset(&g, 0, sizeof(g));
    for (int n = 0; n < NBF; n++)
        for (int e = 0; e < NEQ; e++) Res[n][e] = 0.0;
    for (int ig = 0; ig < NGP; ig++) {
        set_element_basis(G, ig, E);
        basis2d(E, &g);
        set_flow_unknowns(E, &g);                      /* setFlowQuantities :247-262 */
        real_t WiN = strong_form_equations(p, E, &g);
        set_stabilization_terms(p, WiN, E, &g);
        g.WET = (G->w[ig]) * fabs(g.detJ);
        for (int inod = 0; inod < NBF; inod++) {
            real_t term[NEQ];
            for (int e = 0; e < NEQ; e++) term[e] = 0.0;
            momentum_main(p, WiN, E, inod, &g, term);
            continuity_main(E, inod, &g, term);
            stresses_main(p, WiN, E, inod, &g, term);
            for (int e = 0; e < NEQ; e++) Res[inod][e] = Res[inod][e] + term[e] * (g.WET);
        }
    }
}

/* storeBulk :226-313 -- residual and forward-difference Jacobian of one element.
 * The perturbation is restored by subtraction (x + eps) - eps exactly as the
 * Fortran does (:272, :276), so rounding residue carries into later columns. */
static void store_bulk(const prm_t *p, const gauss_t *G, elem_t *E, int want_jac,
                       real_t Res[NBF][NEQ], real_t *A /* [9][6][9][6] */, real_t *Ac /* [9][6][nex] */)
{
    residual_bulk(p, G, E, Res);
    if (!want_jac) return;
    real_t dRes[NBF][NEQ];
    for (int inod = 0; inod < NBF; inod++) {
        for (int ieq = 0; ieq < NEQ; ieq++) {
            real_t eps_jac = p->eps; /* perturbVariableReal, Tools_mod.F90:831-840 */
            E->tl[inod][ieq] = E->tl[inod][ieq] + eps_jac;
            residual_bulk(p, G, E, dRes);
            E->tl[inod][ieq] = E->tl[inod][ieq] - eps_jac;
            for (int jnod = 0; jnod < NBF; jnod++)
                for (int jeq = 0; jeq < NEQ; jeq++)
                    A[((inod * NEQ + ieq) * NBF + jnod) * NEQ + jeq] =
                        (dRes[jnod][jeq] - Res[jnod][jeq]) / eps_jac;
        }
    }
    for (int inex = 0; inex < p->nex; inex++) {
        real_t eps_jac = p->eps;
        E->eu[inex] = E->eu[inex] + eps_jac;
        residual_bulk(p, G, E, dRes);
        E->eu[inex] = E->eu[inex] - eps_jac;
        for (int inod = 0; inod < NBF; inod++)
            for (int ieq = 0; ieq < NEQ; ieq++)
                Ac[(inod * NEQ + ieq) * p->nex + inex] = (dRes[inod][ieq] - Res[inod][ieq]) / eps_jac;
    }
}

#ifndef ORA_COMPLEX_STEP
/* ---------------------------------------------------------------------- */
/* C interface for the tests (ctypes)                                      */

static void unpack_params(const int *ip, const double *dp, prm_t *p)
{
    p->model = ip[0];
    p->form = ip[1];
    p->nex = ip[2];
    p->ReN = dp[0];
    p->WiN = dp[1];
    p->BvN = dp[2];
    p->VeN = dp[3];
    p->DfN = dp[4];
    p->Wi0 = dp[5];
    p->dt = dp[6];
    p->eps = dp[7];
}

/* copyToLocal (Element_Calculations_mod.F90:106-142) from global field-major
 * arrays: TL(Nnodes, Neq) and Xi(Nnodes, 3) column-major, conn(Nel, 9)
 * column-major with 1-based node ids (the reference's own array layouts). */
static void gather_element(int iel, int nel, int nnodes, const int *conn, const double *xyz,
                           const double *TL, const double *EU, int nex, elem_t *E)
{
    memset(E, 0, sizeof(*E));
    for (int inod = 0; inod < NBF; inod++) {
        int g = conn[inod * nel + iel] - 1;
        for (int ieq = 0; ieq < NEQ; ieq++) E->tl[inod][ieq] = TL[(size_t)ieq * nnodes + g];
        for (int j = 0; j < 3; j++) E->xi[inod][j] = xyz[(size_t)j * nnodes + g];
    }
    for (int i = 0; i < nex; i++) E->eu[i] = EU[i];
}

/* Gauss tables for inspection: out[6][9][9] = bfn, dfdc, dfde, d2fdc2, d2fde2, d2fdce; w[9] */
void ora_gauss_tables(double *out, double *w)
{
    gauss_t G;
    gauss_tables(&G);
    memcpy(out + 0 * 81, G.bfn, sizeof(G.bfn));
    memcpy(out + 1 * 81, G.dfdc, sizeof(G.dfdc));
    memcpy(out + 2 * 81, G.dfde, sizeof(G.dfde));
    memcpy(out + 3 * 81, G.d2fdc2, sizeof(G.d2fdc2));
    memcpy(out + 4 * 81, G.d2fde2, sizeof(G.d2fde2));
    memcpy(out + 5 * 81, G.d2fdce, sizeof(G.d2fdce));
    memcpy(w, G.w, sizeof(G.w));
}

/* Element-level outputs for elements [e0, e1):
 *   res[e][9][6]  (Res(inod,ieq))
 *   jac[e][9][6][9][6] (TEMP_A_f(inod,ieq,jnod,jeq)), if jac != NULL
 *   ac[e][9][6][nex]   (TEMP_Ac_f(inod,ieq,inex)),   if jac != NULL and nex > 0 */
int ora_element_batch(const int *ip, const double *dp, int nel, int nnodes, const int *conn,
                      const double *xyz, const double *TL, const double *EU, int e0, int e1,
                      double *res, double *jac, double *ac, int nthreads)
{
    prm_t p;
    unpack_params(ip, dp, &p);
    gauss_t G;
    gauss_tables(&G);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int iel = e0; iel < e1; iel++) {
        elem_t E;
        double Res[NBF][NEQ];
        gather_element(iel, nel, nnodes, conn, xyz, TL, EU, p.nex, &E);
        size_t k = (size_t)(iel - e0);
        store_bulk(&p, &G, &E, jac != NULL, Res, jac ? jac + k * 2916 : NULL,
                   (jac && p.nex > 0) ? ac + k * 54 * p.nex : NULL);
        memcpy(res + k * 54, Res, sizeof(Res));
    }
    (void)nthreads;
    return 0;
}

static long find_slot(const int64_t *rowptr, const int32_t *colind, long row, long col)
{
    long lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        long mid = (lo + hi) / 2;
        if (colind[mid] == col) return mid;
        if (colind[mid] < col) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* setEquationsBulk (Equations_mod.F90:21-55) into a CSR (AIJ) matrix with
 * ADD semantics, element by element in element order, exactly like
 * VecSetValues/MatSetValues(ADD_VALUES) on one rank (Storage_mod.F90:10-115).
 * Element matrices are computed in parallel chunks (nthreads) and added
 * sequentially, so the sums are independent of the thread count.
 * Returns 0, or -1 if an element entry has no slot in the pattern. */
int ora_assemble(const int *ip, const double *dp, int nel, int nnodes, const int *conn,
                 const double *xyz, const double *TL, const double *EU, int want_jac,
                 const int64_t *rowptr, const int32_t *colind, double *b, double *vals,
                 int nthreads)
{
    prm_t p;
    unpack_params(ip, dp, &p);
    const int chunk = 4096;
    double *res = (double *)malloc(sizeof(double) * 54 * chunk);
    double *jac = want_jac ? (double *)malloc(sizeof(double) * 2916 * chunk) : NULL;
    double *ac = (want_jac && p.nex > 0) ? (double *)malloc(sizeof(double) * 54 * p.nex * chunk) : NULL;
    long N = (long)nnodes * NEQ + p.nex;
    int rc = 0;
    for (int e0 = 0; e0 < nel && rc == 0; e0 += chunk) {
        int e1 = e0 + chunk < nel ? e0 + chunk : nel;
        ora_element_batch(ip, dp, nel, nnodes, conn, xyz, TL, EU, e0, e1, res, jac, ac, nthreads);
        for (int iel = e0; iel < e1 && rc == 0; iel++) {
            size_t k = (size_t)(iel - e0);
            long grow1[NBF];
            for (int inod = 0; inod < NBF; inod++)
                grow1[inod] = (long)(conn[inod * nel + iel] - 1) * NEQ; /* getRows - 1 */
            for (int inod = 0; inod < NBF; inod++)                      /* storeResidual */
                for (int ieq = 0; ieq < NEQ; ieq++)
                    b[grow1[inod] + ieq] = b[grow1[inod] + ieq] + res[k * 54 + inod * NEQ + ieq];
            if (!want_jac) continue;
            const double *A = jac + k * 2916;
            for (int jnod = 0; jnod < NBF; jnod++)                      /* storeJacobian */
                for (int jeq = 0; jeq < NEQ; jeq++) {
                    long row = grow1[jnod] + jeq;
                    for (int inod = 0; inod < NBF; inod++)
                        for (int ieq = 0; ieq < NEQ; ieq++) {
                            long s = find_slot(rowptr, colind, row, grow1[inod] + ieq);
                            if (s < 0) { rc = -1; break; }
                            vals[s] = vals[s] + A[((inod * NEQ + ieq) * NBF + jnod) * NEQ + jeq];
                        }
                }
            for (int inex = 0; inex < p.nex; inex++) {                 /* storeJacobian_Ac */
                long col = N - p.nex + inex;
                for (int inod = 0; inod < NBF; inod++)
                    for (int ieq = 0; ieq < NEQ; ieq++) {
                        long s = find_slot(rowptr, colind, grow1[inod] + ieq, col);
                        if (s < 0) { rc = -1; break; }
                        vals[s] = vals[s] + ac[(k * 54 + inod * NEQ + ieq) * p.nex + inex];
                    }
            }
        }
    }
    free(res);
    free(jac);
    free(ac);
    return rc;
}

/* Outlet open-BC edge residual and FD Jacobian of one element edge:
 * residualEdge (Equations_mod.F90:387-424), setEdgeQuantities
 * (Element_Calculations_mod.F90:852-924), openBC (Residuals_mod.F90:599-624),
 * storeEdge (Equations_mod.F90:465-554). ied is 1..4 (eta=-1, xi=+1, eta=+1, xi=-1). */
static void residual_edge_open(const prm_t *p, int ied, elem_t *E, double Res[NBF][NEQ])
{
    double w[3], bfn[3][NBF], dfdc[3][NBF], dfde[3][NBF], d2c[3][NBF], d2e[3][NBF], d2ce[3][NBF];
    gauss_edge_tables(ied, w, bfn, dfdc, dfde, d2c, d2e, d2ce);
    gp_t g;
    memset(&g, 0, sizeof(g));
    for (int n = 0; n < NBF; n++)
        for (int e = 0; e < NEQ; e++) Res[n][e] = 0.0;
    for (int ig = 0; ig < 3; ig++) {
        E->bfn = bfn[ig]; E->dfdc = dfdc[ig]; E->dfde = dfde[ig];
        E->d2fdc2 = d2c[ig]; E->d2fde2 = d2e[ig]; E->d2fdce = d2ce[ig];
        basis2d(E, &g);
        set_flow_unknowns(E, &g);
        double WiN = strong_form_equations(p, E, &g);
        set_stabilization_terms(p, WiN, E, &g);
        double dxdc = g.dXidci[0][0], dydc = g.dXidci[0][1];
        double dxde = g.dXidci[1][0], dyde = g.dXidci[1][1];
        double normal[3] = {0.0, 0.0, 0.0};
        switch (ied) {
        case 1: normal[0] = dydc; normal[1] = -dxdc; break;
        case 2: normal[0] = dyde; normal[1] = -dxde; break;
        case 3: normal[0] = -dydc; normal[1] = dxdc; break;
        default: normal[0] = -dyde; normal[1] = dxde; break;
        }
        double dL = sqrt(normal[0] * normal[0] + normal[1] * normal[1]);
        for (int c = 0; c < 3; c++) normal[c] = normal[c] / dL;
        double WET = w[ig] * dL;
        for (int inod = 0; inod < NBF; inod++) {
            double term[NEQ] = {0, 0, 0, 0, 0, 0};
            double bifn = E->bfn[inod];
            for (int i = 0; i < NEQ_F; i++) {
                double col[3];
                for (int a = 0; a < 3; a++) col[a] = g.P_tot[a][i] + g.P * I3[a][i];
                term[i] = -dot3(normal, col) * bifn;
            }
            for (int e = 0; e < NEQ; e++) Res[inod][e] = Res[inod][e] + term[e] * WET;
        }
    }
}

int ora_edge_open(const int *ip, const double *dp, int nel, int nnodes, const int *conn,
                  const double *xyz, const double *TL, const double *EU, int iel, int ied,
                  double *res, double *jac, double *ac)
{
    prm_t p;
    unpack_params(ip, dp, &p);
    elem_t E;
    double Res[NBF][NEQ], dRes[NBF][NEQ];
    gather_element(iel, nel, nnodes, conn, xyz, TL, EU, p.nex, &E);
    residual_edge_open(&p, ied, &E, Res);
    memcpy(res, Res, sizeof(Res));
    if (!jac) return 0;
    for (int inod = 0; inod < NBF; inod++)
        for (int ieq = 0; ieq < NEQ; ieq++) {
            double eps_jac = p.eps;
            E.tl[inod][ieq] = E.tl[inod][ieq] + eps_jac;
            residual_edge_open(&p, ied, &E, dRes);
            E.tl[inod][ieq] = E.tl[inod][ieq] - eps_jac;
            for (int jnod = 0; jnod < NBF; jnod++)
                for (int jeq = 0; jeq < NEQ; jeq++)
                    jac[((inod * NEQ + ieq) * NBF + jnod) * NEQ + jeq] =
                        (dRes[jnod][jeq] - Res[jnod][jeq]) / eps_jac;
        }
    for (int inex = 0; inex < p.nex; inex++) {
        double eps_jac = p.eps;
        E.eu[inex] = E.eu[inex] + eps_jac;
        residual_edge_open(&p, ied, &E, dRes);
        E.eu[inex] = E.eu[inex] - eps_jac;
        for (int inod = 0; inod < NBF; inod++)
            for (int ieq = 0; ieq < NEQ; ieq++)
                ac[(inod * NEQ + ieq) * p.nex + inex] = (dRes[inod][ieq] - Res[inod][ieq]) / eps_jac;
    }
    return 0;
}

/* Gauss-point strong-form quantities for inspection by the known-answer tests:
 * out = [Momentum(1:2), Continuity, Con_EQ(11,12,22), tlsme, tlsic, tlsce, tdcs, WET] */
int ora_gp_probe(const int *ip, const double *dp, int nel, int nnodes, const int *conn,
                 const double *xyz, const double *TL, const double *EU, int iel, double *out)
{
    prm_t p;
    unpack_params(ip, dp, &p);
    gauss_t G;
    gauss_tables(&G);
    elem_t E;
    gather_element(iel, nel, nnodes, conn, xyz, TL, EU, p.nex, &E);
    gp_t g;
    memset(&g, 0, sizeof(g));
    for (int ig = 0; ig < NGP; ig++) {
        set_element_basis(&G, ig, &E);
        basis2d(&E, &g);
        set_flow_unknowns(&E, &g);
        double WiN = strong_form_equations(&p, &E, &g);
        set_stabilization_terms(&p, WiN, &E, &g);
        g.WET = (G.w[ig]) * fabs(g.detJ);
        double *o = out + ig * 11;
        o[0] = g.Momentum[0]; o[1] = g.Momentum[1]; o[2] = g.Continuity;
        o[3] = g.Con_EQ[0][0]; o[4] = g.Con_EQ[0][1]; o[5] = g.Con_EQ[1][1];
        o[6] = g.tlsme; o[7] = g.tlsic; o[8] = g.tlsce; o[9] = g.tdcs; o[10] = g.WET;
    }
    return 0;
}
#endif /* !ORA_COMPLEX_STEP */

#ifdef ORA_COMPLEX_STEP
static void cs_unpack_params(const int *ip, const double *dp, prm_t *p)
{
    p->model = ip[0];
    p->form = ip[1];
    p->nex = ip[2];
    p->ReN = dp[0];
    p->WiN = dp[1];
    p->BvN = dp[2];
    p->VeN = dp[3];
    p->DfN = dp[4];
    p->Wi0 = dp[5];
    p->dt = dp[6];
    p->eps = dp[7];
}

/* Exact element Jacobians by the complex step, elements [e0, e1), in the
 * layouts of ora_element_batch: res[e][9][6], jac[e][9][6][9][6]
 * (d Res(jnod,jeq) / d TL(inod,ieq) at [inod][ieq][jnod][jeq]) and
 * ac[e][9][6][nex] (d Res(inod,ieq) / d EU(inex)). */
int ora_cs_element_batch(const int *ip, const double *dp, int nel, int nnodes, const int *conn,
                         const double *xyz, const double *TL, const double *EU, int e0, int e1,
                         double *res, double *jac, double *ac, int nthreads)
{
    const double h = 1.0e-30;
    prm_t p;
    cs_unpack_params(ip, dp, &p);
    gauss_t G;
    gauss_tables(&G);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int iel = e0; iel < e1; iel++) {
        elem_t E;
        real_t Res[NBF][NEQ], dRes[NBF][NEQ];
        memset(&E, 0, sizeof(E));
        for (int inod = 0; inod < NBF; inod++) {
            int g = conn[inod * nel + iel] - 1;
            for (int ieq = 0; ieq < NEQ; ieq++) E.tl[inod][ieq] = TL[(size_t)ieq * nnodes + g];
            for (int j = 0; j < 3; j++) E.xi[inod][j] = xyz[(size_t)j * nnodes + g];
        }
        for (int i = 0; i < p.nex; i++) E.eu[i] = EU[i];
        size_t k = (size_t)(iel - e0);
        residual_bulk(&p, &G, &E, Res);
        for (int inod = 0; inod < NBF; inod++)
            for (int ieq = 0; ieq < NEQ; ieq++) res[k * 54 + inod * NEQ + ieq] = creal(Res[inod][ieq]);
        for (int inod = 0; inod < NBF; inod++)
            for (int ieq = 0; ieq < NEQ; ieq++) {
                const double x0 = creal(E.tl[inod][ieq]);
                E.tl[inod][ieq] = CMPLX(x0, h);
                residual_bulk(&p, &G, &E, dRes);
                E.tl[inod][ieq] = x0;
                for (int jnod = 0; jnod < NBF; jnod++)
                    for (int jeq = 0; jeq < NEQ; jeq++)
                        jac[k * 2916 + ((inod * NEQ + ieq) * NBF + jnod) * NEQ + jeq] =
                            cimag(dRes[jnod][jeq]) / h;
            }
        for (int inex = 0; inex < p.nex; inex++) {
            const double x0 = creal(E.eu[inex]);
            E.eu[inex] = CMPLX(x0, h);
            residual_bulk(&p, &G, &E, dRes);
            E.eu[inex] = x0;
            for (int inod = 0; inod < NBF; inod++)
                for (int ieq = 0; ieq < NEQ; ieq++)
                    ac[(k * 54 + inod * NEQ + ieq) * p.nex + inex] = cimag(dRes[inod][ieq]) / h;
        }
    }
    (void)nthreads;
    return 0;
}
#endif /* ORA_COMPLEX_STEP */
