/*
 * vefem_stability_oracle.c -- CPU oracle of the linear-stability assembly
 * (generalised eigenproblem A x = lambda B x for spanwise-periodic 3-D
 * perturbations of a 2-D base flow).
 *
 * TEST INFRASTRUCTURE ONLY, like vefem_oracle.c, which it includes: only the
 * tests load it; the product never links or calls it.
 *
 * Restated routines (Stability/ directory of the reference):
 *   setEquationsBulkStability / residualBulkStability / storeBulkStability
 *     (Equations_Stability_mod.F90:20-226): per element Res_a, Res_b and the
 *     forward-difference blocks TEMP_A_f, TEMP_B_f (absolute eps 1e-8, the
 *     perturbation restored by subtraction);
 *   setFlowQuantitiesStability (Element_Calculations_Stability_mod.F90:19-102)
 *     with setFlowUnknownsStabilityReal (:106-173), strongFormMomentumStability
 *     (:315-341) and setExtraFlowUnknownsStability (:280-311, the real
 *     sin/cos split, Stability_Im = .false.);
 *   strongFormConEQ_Stability, conEQ_*_Stability, setUCDStability,
 *     setStressTensorStability (Constitutive_Models_Stability_mod.F90, T form;
 *     L-PTT, m-L-PTT, e-PTT, m-e-PTT and Giesekus);
 *   momentumStabilityT / momentumStability3D / continuityStability /
 *     stressStabilityT (Residuals_Stability_mod.F90:34-210);
 *   the base state embedding of updateStabilityArrays
 *     (Continuation_Stability_mod.F90:592-633): [Ux, Uy, 0, P, Txx, Txy, Tyy, 0, 0, 0].
 * The base quantities use the stability problem's dimension N = 3 in the
 * traceless kinematics (setFlowKinematics(Problem_Stability%Ndim)).
 *
 * Unknowns per node (Neq = 10): Ux, Uy, Uz, P, Txx, Txy, Tyy, Txz, Tyz, Tzz.
 *
 * The reference's path is incomplete: the z-derivative terms of the
 * perturbation are commented out in setFlowQuantitiesStability (:52-79), so
 * only momentumStability3D sees the wavenumber.  With kz = 1 this oracle
 * restates the intended equations (setExtraFlowUnknownsStability applied);
 * kz = 0 follows the source as written.  Parity unpinned: the reference
 * cannot be built here and ships no stability data; the oracle is pinned by
 * the linearity of the perturbation residual, its k-dependence, and
 * B-matrix identities in the tests.
 */
#include "vefem_oracle.c"

#define NEQ_ST 10
#define NEQF_ST 3
#define NEQS_ST 6

typedef struct {
    double tlb[NBF][NEQ_ST];   /* base, TEMP_TL_b */
    double tld[NBF][NEQ_ST];   /* perturbation, TEMP_TL_d */
} stab_elem_t;

/* setFlowUnknownsStabilityReal :106-173 */
static void set_flow_unknowns_stab(const elem_t *E, const double tl[NBF][NEQ_ST], gp_t *g)
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
    for (int i = 0; i < NEQF_ST; i++) {
        g->U_f[i] = dot9(&tl[0][i], NEQ_ST, E->bfn);
        for (int j = 0; j < 3; j++) {
            g->GU[j][i] = dot9(&tl[0][i], NEQ_ST, E->dFdXi[j]);
            g->G2U[j][i] = dot9(&tl[0][i], NEQ_ST, E->d2FdXi2[j]);
        }
        g->dPdXi[i] = dot9(&tl[0][NEQF_ST], NEQ_ST, E->dFdXi[i]);
    }
    g->P = dot9(&tl[0][NEQF_ST], NEQ_ST, E->bfn);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            g->S[a][b] = 0.0;
            for (int c = 0; c < 3; c++) g->dSdXi[a][b][c] = 0.0;
        }
    const int istart = NEQ_ST - NEQS_ST;
    for (int i = istart; i < NEQ_ST; i++) {
        int j, k;
        stress_component(i, istart, &j, &k);
        g->S[j][k] = dot9(&tl[0][i], NEQ_ST, E->bfn);
        g->S[k][j] = g->S[j][k];
        for (int idim = 0; idim < 3; idim++)
            g->dSdXi[j][k][idim] = dot9(&tl[0][i], NEQ_ST, E->dFdXi[idim]);
        for (int idim = 0; idim < 3; idim++) g->dSdXi[k][j][idim] = g->dSdXi[j][k][idim];
    }
}

/* setFlowKinematics (Element_Calculations_mod.F90:605-634) with dimension N */
static void set_flow_kinematics_n(gp_t *g, int N)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GUT[i][j] = g->GU[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->G_dot[i][j] = g->GU[i][j] + g->GUT[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GU_tr[i][j] = g->GU[i][j];
    double tr = trace3(g->GU);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) g->GU_tr[i][j] = g->GU[i][j] - tr * I3[i][j] / (double)N;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->GUT_tr[i][j] = g->GU_tr[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) g->G_dot_tr[i][j] = g->GU_tr[i][j] + g->GUT_tr[i][j];
}

/* setExtraFlowUnknownsStability :280-311, Stability_Im = .false.: the
 * perturbation is u, v, p, Txx, Txy, Tyy, Tzz ~ cos(kz) and w, Txz, Tyz ~ sin(kz) */
static void extra_flow_unknowns_stab(gp_t *g, double KwN)
{
    const int N = 2;   /* z, 0-based */
    g->GU[N][0] = -KwN * (g->U_f[0]);
    g->GU[N][1] = -KwN * (g->U_f[1]);
    g->GU[N][N] = KwN * (g->U_f[N]);
    g->dPdXi[N] = -KwN * g->P;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) g->dSdXi[a][b][N] = -KwN * g->S[a][b];
    g->dSdXi[0][N][N] = KwN * g->S[0][N];
    g->dSdXi[N][0][N] = g->dSdXi[0][N][N];
    g->dSdXi[1][N][N] = KwN * g->S[1][N];
    g->dSdXi[N][1][N] = g->dSdXi[1][N][N];
    for (int i = 0; i < 3; i++) g->G2U[N][i] = -(KwN * KwN) * g->U_f[i];
}

/* setFENEMaterialDerivativeStability (Constitutive_Models_Stability_mod.F90:294-328):
 * the perturbation of U . grad f_T, with grad f_T from the trace of grad T */
static double fene_md_stab(const prm_t *p, double WiN, const gp_t *b, const gp_t *d)
{
    double dfb[3] = {0.0, 0.0, 0.0}, dfd[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) {
            dfb[c] = dfb[c] + b->dTdXi[i][i][c];
            dfd[c] = dfd[c] + d->dTdXi[i][i][c];
        }
    const double den = (p->model == M_FENE_P) ? p->VeN : (p->VeN - (double)NDIM);
    for (int c = 0; c < 3; c++) {
        dfb[c] = (WiN / (1.0 - p->BvN)) * dfb[c] / den;
        dfd[c] = (WiN / (1.0 - p->BvN)) * dfd[c] / den;
    }
    double MD = 0.0;
    for (int i = 0; i < 3; i++) {
        const double term = ((b->f_T) * dfd[i] - (d->f_T) * dfb[i]) / (b->f_T);
        MD = MD + (d->U_f[i]) * dfb[i] + (b->U_f[i]) * term;
    }
    return MD;
}

/* conEQ_*_Stability (Constitutive_Models_Stability_mod.F90:96-289) */
static int con_eq_T_stab(const prm_t *p, double WiN, const gp_t *b, gp_t *d)
{
    double trT_d = trace3(d->S);
    double ePTT = p->VeN, BvN = p->BvN;
    switch (p->model) {
    case M_L_PTT:
        d->f_T = ePTT * WiN * trT_d / (1.0 - BvN);
        d->f[0] = 0.0; d->f[1] = d->f_T; d->f[2] = 0.0;
        d->g[0] = 0.0; d->g[1] = 0.0;
        return 0;
    case M_M_L_PTT:
        d->f_T = ePTT * WiN * trT_d / (1.0 - BvN);
        d->f[0] = d->f_T; d->f[1] = d->f[0]; d->f[2] = 0.0;
        d->g[0] = d->f_T; d->g[1] = d->g[0];
        return 0;
    case M_E_PTT:
        d->f_T = (b->f_T) * ePTT * WiN * trT_d / (1.0 - BvN);
        d->f[0] = 0.0; d->f[1] = d->f_T; d->f[2] = 0.0;
        d->g[0] = 0.0; d->g[1] = 0.0;
        return 0;
    case M_M_E_PTT:
        d->f_T = (b->f_T) * ePTT * WiN * trT_d / (1.0 - BvN);
        d->f[0] = d->f_T; d->f[1] = d->f[0]; d->f[2] = 0.0;
        d->g[0] = d->f_T; d->g[1] = d->g[0];
        return 0;
    case M_GIESEKUS:
        d->f_T = 0.0;
        d->f[0] = 0.0; d->f[1] = 0.0; d->f[2] = 0.0;
        d->g[0] = 0.0; d->g[1] = 0.0;
        return 0;
    case M_FENE_CR: {   /* :236-260, N = Ndim of the base problem */
        d->f_T = (WiN * trT_d / (1.0 - BvN)) / (p->VeN - (double)NDIM);
        d->f[0] = d->f_T;
        const double MD = fene_md_stab(p, WiN, b, d);
        d->f[1] = d->f_T - WiN * MD / (b->f_T);
        d->f[2] = 0.0;
        d->g[0] = d->f_T; d->g[1] = d->g[0];
        return 0;
    }
    case M_FENE_P: {    /* :264-289 */
        d->f_T = (WiN * trT_d / (1.0 - BvN)) / p->VeN;
        d->f[0] = 0.0;
        const double MD = fene_md_stab(p, WiN, b, d);
        d->f[1] = d->f_T - WiN * MD / (b->f_T);
        d->f[2] = 0.0;
        d->g[0] = 0.0; d->g[1] = d->f_T;
        return 0;
    }
    default:
        return -1;
    }
}

/* Con_EQ_time of the perturbation (strongFormConEQ_Stability :85-93) */
static void con_eq_time_stab(const prm_t *p, double WiN, const gp_t *b, const gp_t *d,
                             double ceqt[3][3])
{
    double term_I = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) ceqt[i][j] = WiN * (d->S[i][j]);
    if (p->model == M_FENE_CR || p->model == M_FENE_P) {
        if (p->model == M_FENE_P) term_I = -(1.0 - p->BvN) * (d->f_T) / (b->f_T);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                ceqt[i][j] = ceqt[i][j] - WiN * (d->f_T) * b->S[i][j] / (b->f_T);
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) ceqt[i][j] = ceqt[i][j] + term_I * I3[i][j];
}

/* strongFormConEQ_Stability :55-94 with setUCDStability :330-351 and
 * setStressTensorStability :355-371 (T form) */
static void strong_form_con_eq_T_stab(const prm_t *p, double WiN, const gp_t *b, gp_t *d)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            d->T_ve[i][j] = d->S[i][j];
            for (int k = 0; k < 3; k++) d->dTdXi[i][j][k] = d->dSdXi[i][j][k];
        }
    con_eq_T_stab(p, WiN, b, d);
    /* setStressTensorStability */
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            d->P_tot[i][j] = d->T_ve[i][j] + p->BvN * (d->G_dot[i][j]) - (d->P) * I3[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            d->C_Tensor[i][j] = WiN * (d->T_ve[i][j] / (1.0 - p->BvN)) + d->g[0] * I3[i][j]
                                - (d->g[1]) * (b->C_Tensor[i][j]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) d->C_Tensor[i][j] = (1.0 / (b->g[1])) * (d->C_Tensor[i][j]);
    /* setUCDStability */
    double UCD[3][3], M1[3][3], M2[3][3], M3[3][3], M4[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = 0.0;
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                UCD[i][j] = UCD[i][j] + (b->U_f[k]) * (d->dTdXi[i][j][k])
                            + (d->U_f[k]) * (b->dTdXi[i][j][k]);
    matmul3(b->GUT, d->S, M1);
    matmul3(d->GUT, b->S, M2);
    matmul3(b->S, d->GU, M3);
    matmul3(d->S, b->GU, M4);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) UCD[i][j] = UCD[i][j] - M1[i][j] - M2[i][j] - M3[i][j] - M4[i][j];
    /* term_I of FENE-P */
    double term_I = 0.0;
    if (p->model == M_FENE_P) term_I = fene_md_stab(p, WiN, b, d) / (b->f_T);
    /* term_T */
    double SbSd[3][3], SdSb[3][3], SbSb[3][3];
    matmul3(b->S, d->S, SbSd);
    matmul3(d->S, b->S, SdSb);
    matmul3(b->S, b->S, SbSb);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double term_T = (b->f[2]) * (SbSd[i][j] + SdSb[i][j]) + (d->f[2]) * SbSb[i][j]
                            + (d->f[1]) * b->S[i][j] + (b->f[1]) * d->S[i][j];
            double term_G = (b->f[0]) * (d->G_dot[i][j]) + (d->f[0]) * (b->G_dot[i][j]);
            d->Con_EQ[i][j] = WiN * UCD[i][j] + term_T - (1.0 - p->BvN) * (term_G + term_I * I3[i][j]);
        }
}

/* strongFormMomentumStability :315-341; returns Momentum_time in mt */
static void strong_form_momentum_stab(const prm_t *p, const gp_t *b, gp_t *d, double mt[3])
{
    double div_Tve[3] = {0.0, 0.0, 0.0}, div_Ptot[3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) div_Tve[i] = div_Tve[i] + d->dTdXi[j][i][j];
    for (int i = 0; i < 3; i++)
        div_Ptot[i] = -d->dPdXi[i] + div_Tve[i]
                      + p->BvN * ((d->G2U[0][i]) + (d->G2U[1][i]) + (d->G2U[2][i]));
    for (int i = 0; i < 3; i++) {
        double s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < 3; k++) s1 = s1 + b->U_f[k] * d->GU[k][i];
        for (int k = 0; k < 3; k++) s2 = s2 + d->U_f[k] * b->GU[k][i];
        d->Convection[i] = s1 + s2;
    }
    for (int i = 0; i < 3; i++) {
        d->Momentum[i] = p->ReN * (d->Convection[i]) - div_Ptot[i];
        mt[i] = p->ReN * (d->U_f[i]);
    }
}

/* residualBulkStability :60-97 with equationsResidualsBulkStability :101-135 */
static void residual_bulk_stab(const prm_t *p, double WiN, double KwN, int kz, const gauss_t *G,
                               elem_t *E, const stab_elem_t *S, double Ra[NBF][NEQ_ST],
                               double Rb[NBF][NEQ_ST])
{
    gp_t gb, gd;
    memset(&gb, 0, sizeof(gb));
    memset(&gd, 0, sizeof(gd));
    for (int n = 0; n < NBF; n++)
        for (int e = 0; e < NEQ_ST; e++) {
            Ra[n][e] = 0.0;
            Rb[n][e] = 0.0;
        }
    for (int ig = 0; ig < NGP; ig++) {
        set_element_basis(G, ig, E);
        basis2d(E, &gb);
        /* base: setFlowUnknownsStability, strongFormEquations(Problem_Stability),
         * setStabilizationTerms */
        set_flow_unknowns_stab(E, S->tlb, &gb);
        set_flow_kinematics_n(&gb, 3);
        for (int i = 0; i < 3; i++) {
            gb.dUfdt[i] = 0.0;
            for (int j = 0; j < 3; j++) gb.dSdt[i][j] = 0.0;
        }
        strong_form_con_eq_T(p, WiN, &gb);
        strong_form_momentum(p, &gb);
        gb.Continuity = trace3(gb.GU);
        set_stabilization_terms(p, WiN, E, &gb);
        /* perturbation */
        set_flow_unknowns_stab(E, S->tld, &gd);
        if (kz) extra_flow_unknowns_stab(&gd, KwN);
        set_flow_kinematics_n(&gd, 3);
        strong_form_con_eq_T_stab(p, WiN, &gb, &gd);
        double mt[3];
        strong_form_momentum_stab(p, &gb, &gd, mt);
        gd.Continuity = trace3(gd.GU);     /* strongFormContinuity */
        double ceqt[3][3];                 /* Con_EQ_time */
        con_eq_time_stab(p, WiN, &gb, &gd, ceqt);
        gd.mag_con_EQ = ddot3(gb.Con_EQ, gd.Con_EQ);
        gd.mag_con_EQ = gd.mag_con_EQ / (2.0 * gb.mag_con_EQ + 1.0e-12);
        /* the steady base has Con_EQ_time = 0, so mag_con_EQ_time of the
         * perturbation is 0 / (0 + 1e-12) = 0 */
        const double mag_time = 0.0;
        gb.WET = (G->w[ig]) * fabs(gb.detJ);

        for (int inod = 0; inod < NBF; inod++) {
            double ta[NEQ_ST], tb[NEQ_ST];
            for (int e = 0; e < NEQ_ST; e++) {
                ta[e] = 0.0;
                tb[e] = 0.0;
            }
            const double bifn = E->bfn[inod];
            const double dF[3] = {E->dFdXi[0][inod], E->dFdXi[1][inod], E->dFdXi[2][inod]};
            /* momentumStabilityT :34-82 */
            for (int i = 0; i < NEQF_ST; i++) {
                double lsme_term = (gb.tlsme) * p->ReN * dot3(gb.U_f, dF);   /* LSMEMomentum */
                double lsic_term = gb.tlsic * dF[i];                          /* LSICMomentum */
                lsic_term = lsic_term * (gd.Continuity);
                double lsce[3][3];                                            /* LSCEMomentumT */
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) lsce[a][c] = -gb.tlsce * (a == i ? dF[c] : 0.0);
                double lsce_term = ddot3(lsce, gd.Con_EQ);
                double Pi[3] = {gd.P_tot[i][0], gd.P_tot[i][1], gd.P_tot[i][2]};
                ta[i] = p->ReN * (gd.Convection[i]) * bifn + dot3(Pi, dF)
                        + lsme_term * (gd.Momentum[i]) + lsic_term + lsce_term;
                lsce_term = ddot3(lsce, ceqt);
                tb[i] = mt[i] * bifn + lsme_term * (mt[i]) + lsce_term;
            }
            /* momentumStability3D :86-115 (real split) */
            for (int i = 0; i < 3; i++) {
                double term = bifn * KwN;
                if (i == 2) term = -term;
                ta[i] = ta[i] - term * (gd.P_tot[i][2]);
            }
            /* continuityStability :119-144 */
            {
                double lsme_term = gb.tlsme * dot3(dF, gd.Momentum);
                ta[NEQF_ST] = (gd.Continuity) * bifn + lsme_term;
                lsme_term = gb.tlsme * dot3(dF, mt);
                tb[NEQF_ST] = lsme_term;
            }
            /* stressStabilityT :148-188 */
            const int istart = NEQ_ST - NEQS_ST;
            for (int ii = istart; ii < NEQ_ST; ii++) {
                int j, k;
                stress_component(ii, istart, &j, &k);
                double lsme_term = -dF[k] * gd.Momentum[j];            /* LSMEStressT */
                if (j != k) lsme_term = lsme_term - dF[j] * gd.Momentum[k];
                lsme_term = gb.tlsme * lsme_term * (1.0 - p->BvN);
                double lsce_term = WiN * dot3(gb.U_f, dF);            /* LSCEStressT */
                lsce_term = (gb.tlsce) * lsce_term;
                double dcs_term = (gb.tdcs) * dot3(gb.dTdXi[j][k], dF); /* DCSStressT */
                ta[ii] = (gd.Con_EQ[j][k]) * bifn + p->DfN * dot3(gd.dTdXi[j][k], dF)
                         + lsme_term + lsce_term * (gd.Con_EQ[j][k]) + dcs_term * (gd.mag_con_EQ);
                lsme_term = -dF[k] * mt[j];
                if (j != k) lsme_term = lsme_term - dF[j] * mt[k];
                lsme_term = gb.tlsme * lsme_term * (1.0 - p->BvN);
                tb[ii] = (ceqt[j][k]) * bifn + lsme_term + lsce_term * (ceqt[j][k])
                         + dcs_term * mag_time;
            }
            for (int e = 0; e < NEQ_ST; e++) {
                tb[e] = -tb[e];
                Ra[inod][e] = Ra[inod][e] + ta[e] * (gb.WET);
                Rb[inod][e] = Rb[inod][e] + tb[e] * (gb.WET);
            }
        }
    }
}

/* storeBulkStability :139-226 without the extra unknowns (Nex = 0) */
static void store_bulk_stab(const prm_t *p, double WiN, double KwN, int kz, const gauss_t *G,
                            elem_t *E, stab_elem_t *S, double Ra[NBF][NEQ_ST],
                            double Rb[NBF][NEQ_ST], double *A, double *B)
{
    residual_bulk_stab(p, WiN, KwN, kz, G, E, S, Ra, Rb);
    if (!A) return;
    double dRa[NBF][NEQ_ST], dRb[NBF][NEQ_ST];
    for (int inod = 0; inod < NBF; inod++)
        for (int ieq = 0; ieq < NEQ_ST; ieq++) {
            const double eps_jac = p->eps;   /* perturbVariableReal */
            S->tld[inod][ieq] = S->tld[inod][ieq] + eps_jac;
            residual_bulk_stab(p, WiN, KwN, kz, G, E, S, dRa, dRb);
            S->tld[inod][ieq] = S->tld[inod][ieq] - eps_jac;
            for (int jnod = 0; jnod < NBF; jnod++)
                for (int jeq = 0; jeq < NEQ_ST; jeq++) {
                    const size_t o = (((size_t)inod * NEQ_ST + ieq) * NBF + jnod) * NEQ_ST + jeq;
                    A[o] = (dRa[jnod][jeq] - Ra[jnod][jeq]) / eps_jac;
                    B[o] = (dRb[jnod][jeq] - Rb[jnod][jeq]) / eps_jac;
                }
        }
}

/* Element outputs of the stability assembly for elements [e0, e1):
 *   ra[e][9][10], rb[e][9][10] (Res_a, Res_b at the perturbation TLd)
 *   A[e][9][10][9][10], B[...] (TEMP_A_f(inod,ieq,jnod,jeq), TEMP_B_f), if A != NULL.
 * TLb: base [10][nnodes] field-major (the embedded 2-D base); TLd likewise.
 * ip = [model, form, nex], dp as ora_element_batch (WiN = dp[1]). */
int ora_stability_batch(const int *ip, const double *dp, double KwN, int kz, int nel, int nnodes,
                        const int *conn, const double *xyz, const double *TLb, const double *TLd,
                        int e0, int e1, double *ra, double *rb, double *A, double *B, int nthreads)
{
    prm_t p;
    unpack_params(ip, dp, &p);
    if (p.form != FORM_T) return -2;

    gauss_t G;
    gauss_tables(&G);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int iel = e0; iel < e1; iel++) {
        elem_t E;
        stab_elem_t S;
        memset(&E, 0, sizeof(E));
        for (int inod = 0; inod < NBF; inod++) {
            const int g = conn[inod * nel + iel] - 1;
            for (int j = 0; j < 3; j++) E.xi[inod][j] = xyz[(size_t)j * nnodes + g];
            for (int q = 0; q < NEQ_ST; q++) {
                S.tlb[inod][q] = TLb[(size_t)q * nnodes + g];
                S.tld[inod][q] = TLd[(size_t)q * nnodes + g];
            }
        }
        double Ra[NBF][NEQ_ST], Rb[NBF][NEQ_ST];
        const size_t k = (size_t)(iel - e0);
        const size_t blk = (size_t)NBF * NEQ_ST * NBF * NEQ_ST;
        store_bulk_stab(&p, p.WiN, KwN, kz, &G, &E, &S, Ra, Rb, A ? A + k * blk : NULL,
                        B ? B + k * blk : NULL);
        memcpy(ra + k * NBF * NEQ_ST, Ra, sizeof(Ra));
        memcpy(rb + k * NBF * NEQ_ST, Rb, sizeof(Rb));
    }
    (void)nthreads;
    return 0;
}
