// tables.cpp -- host-side potential registry and force-table generator.
//
// The reference builds its tables on the host once per run (Register_Interaction_Table ->
// Create_Interaction_ForceTable, MD_TypeDef_ForceTable.F90:1151-1230) and uploads them in
// INITIALIZE_*_Force_Table_DEV.  This file is the library's C++ equivalent for the three
// potentials the hot path is benchmarked with, in Angstrom / eV:
//   Cleri-Rosato TB-SMA (TB_CR_AuAu.F90:22-56 form, any parameter set; FS type)
//   Marinica EAM2 W (EAM2_WW_Marinica_JPCM25_2013.F90:17-116 with the cubic-knot helpers
//                    MD_Pot_EAM_Utilities.F90:48-85, 259-290, 332-368; EAM type)
//   Ackland-Thetford W (FS_Ackland_WW.F90:23-88; FS type)
// Grid (Create_Pairwise_ForceTable :949-976): T = i*CSIV, R = T*T, CSI = NTAB/sqrt(Rmax);
// POTR = f1(R)*R, FPOTR = f2(R)*R, POTB = rho(R), FPOTB = -rho'(R);
// RHOMX = RHOSCAL * max POTB, RHOD = RHOMX/NEMBD; F, F' at rho = (i-1)*RHOD (:1040-1048).
#include <cmath>

#include "../../include/msmgb.h"

namespace {

struct PairVal {
    double potr, fpotr, potb, fpotb;
};

// Cleri-Rosato: V = A exp(-p(r/r0-1)) with FPOTR = 2 V p/r0; rho = xi^2 exp(-2q(r/r0-1))
// with FPOTB = rho q/r0 * 2.
PairVal cleri_rosato(double r, const double *prm)
{
    const double A = prm[0], xi = prm[1], P = prm[2], Q = prm[3], r0 = prm[4];
    PairVal o;
    o.potr = A * std::exp(-P * ((r / r0) - 1.0));
    o.fpotr = 2.0 * o.potr * (P / r0);
    o.potb = (xi * xi) * std::exp(-(2.0 * Q) * ((r / r0) - 1.0));
    o.fpotb = o.potb * (Q / r0) * 2.0;
    return o;
}

// Marinica EAM2.  The knot radii are single-precision literals in the reference source, so
// their values are the float roundings of the printed decimals.
const double kMarA[15] = {0.960851701343041e2, -0.184410923895214e3, 0.935784079613550e2,
                          -0.798358265041677e1, 0.747034092936229e1, -0.152756043708453e1,
                          0.125205932634393e1, 0.163082162159425e1, -0.141854775352260e1,
                          -0.819936046256149e0, 0.198013514305908e1, -0.696430179520267e0,
                          0.304546909722160e-1, -0.163131143161660e1, 0.138409896486177e1};
const float kMarR[15] = {2.5648975f, 2.629795f, 2.6946925f, 2.8663175f, 2.973045f,
                         3.0797725f, 3.5164725f, 3.846445f, 4.1764175f, 4.700845f,
                         4.8953f, 5.089755f, 5.3429525f, 5.401695f, 5.4604375f};
const double kMarB[4] = {-0.420429107805055e1, 0.518217702261442e0, 0.562720834534370e-1,
                         0.344164178842340e-1};
const float kMarRB[4] = {2.5f, 3.1f, 3.5f, 4.9f};
const double kMarRC = 2.002970124727;
const double kMarF[2] = {-5.946454472402710, -0.049477376935239};

void cubic_knots(double rt, const double *a, const float *ri, int n, double *v, double *f)
{
    double p = 0.0, d = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = (double)ri[i];
        double stp = (r - rt) >= 0.0 ? 1.0 : 0.0;
        p = p + a[i] * (r - rt) * (r - rt) * (r - rt) * stp;
        d = d + a[i] * (r - rt) * (r - rt) * stp;
    }
    *v = p;
    *f = 3.0 * d;
}

PairVal marinica2(double r)
{
    PairVal o;
    double v, f;
    cubic_knots(r, kMarA, kMarR, 15, &v, &f);
    o.potr = 0.5 * v;            // NN_FuncPoly3 returns 0.5 V and -V'
    o.fpotr = f;
    if (r <= kMarRC) {           // density frozen inside RC
        cubic_knots(kMarRC, kMarB, kMarRB, 4, &o.potb, &o.fpotb);
        o.fpotb = 0.0;
    } else {
        cubic_knots(r, kMarB, kMarRB, 4, &o.potb, &o.fpotb);
    }
    return o;
}

void marinica2_embed(double rho, double *f, double *df)
{
    if (rho <= 0.0) { *f = 0.0; *df = 0.0; return; }
    *f = kMarF[0] * std::sqrt(rho) + kMarF[1] * rho * rho;
    *df = 0.5 * kMarF[0] / std::sqrt(rho) + 2.0 * kMarF[1] * rho;
}

PairVal ackland_ww(double r)
{
    const double c = 3.25, c0 = 47.1346499, c1 = -33.7665655, c2 = 6.2541999;
    const double ackb = 90.3, acka = 1.2, ackb0 = 2.7411, a = 1.896373, d = 4.400224;
    PairVal o{0.0, 0.0, 0.0, 0.0};
    double fs = 0.0, dfs = 0.0;
    if (r < ackb0) {
        double t = ackb0 - r, e = std::exp(-acka * r);
        fs = ackb * t * t * t * e;
        dfs = -ackb * (3.0 * t * t * e + acka * t * t * t * e);
    }
    if (r <= c) {
        double poly = c0 + c1 * r + c2 * r * r;
        o.potr = 0.5 * ((r - c) * (r - c) * poly + fs);
        o.fpotr = -(2.0 * (r - c) * poly + (r - c) * (r - c) * (c1 + 2.0 * c2 * r) + dfs);
    }
    if (r <= d) {
        o.potb = a * a * (r - d) * (r - d);
        o.fpotb = -(a * a * 2.0 * (r - d));
    }
    return o;
}

}  // namespace

extern "C" int msmgb_create_forcetable(int pot, const double *prm, double rmax, int ntab,
                                       int nembd, double rhoscal, double *potr, double *fpotr,
                                       double *potb, double *fpotb, double *fembd,
                                       double *dfembd, double *rhod)
{
    if (ntab < 2 || rmax <= 0.0 || !potr || !fpotr || !potb || !fpotb) return MSMGB_ERR_ARG;
    if (pot == MSMGB_POT_CR && !prm) return MSMGB_ERR_ARG;
    if (pot != MSMGB_POT_CR && pot != MSMGB_POT_MARINICA2 && pot != MSMGB_POT_ACKLAND_WW)
        return MSMGB_ERR_ARG;
    const double csi = (double)ntab / std::sqrt(rmax);
    const double csiv = 1.0 / csi;
    double rhomx = -1.0;
    for (int i = 1; i <= ntab; ++i) {
        double t = (double)i * csiv;
        double r = t * t;
        PairVal v = pot == MSMGB_POT_CR ? cleri_rosato(r, prm)
                  : pot == MSMGB_POT_MARINICA2 ? marinica2(r) : ackland_ww(r);
        potr[i - 1] = v.potr * r;
        fpotr[i - 1] = v.fpotr * r;
        potb[i - 1] = v.potb;
        fpotb[i - 1] = v.fpotb;
        if (rhomx < v.potb * rhoscal) rhomx = v.potb * rhoscal;
    }
    double rd = nembd > 0 ? rhomx / (double)nembd : 0.0;
    if (rhod) *rhod = rd;
    if (fembd && dfembd && nembd > 0) {
        for (int i = 1; i <= nembd; ++i) {
            double rho = (double)(i - 1) * rd;
            if (pot == MSMGB_POT_MARINICA2) {
                marinica2_embed(rho, &fembd[i - 1], &dfembd[i - 1]);
            } else {
                fembd[i - 1] = 0.0;
                dfembd[i - 1] = 0.0;
            }
        }
    }
    return MSMGB_OK;
}

// Derivatives of the Cleri-Rosato pair tables with respect to theta = (A, xi, p, q, r0), on the
// same sqrt(r) grid, for the force-matching adjoint.  With a = r/r0 - 1, V = A exp(-p a),
// rho = xi^2 exp(-2 q a):
//   FPOTR = 2 V p r / r0:  d/dA = FPOTR/A,  d/dp = 2 r V (1 - p a)/r0,
//                          d/dr0 = 2 p r V (p r/r0 - 1)/r0^2
//   POTB  = rho:           d/dxi = 2 rho/xi, d/dq = -2 a rho, d/dr0 = 2 q r rho/r0^2
//   FPOTB = 2 q rho/r0:    d/dxi = 2 FPOTB/xi, d/dq = 2 rho (1 - 2 q a)/r0,
//                          d/dr0 = 2 q rho (2 q r/r0 - 1)/r0^2
// Output layout: d[(m*3 + t)*ntab + (i-1)] for parameter m = 0..4 and table t = 0 (FPOTR),
// 1 (POTB), 2 (FPOTB).
extern "C" int msmgb_cr_param_tables(const double *prm, double rmax, int ntab, double *d)
{
    if (!prm || !d || ntab < 2 || rmax <= 0.0) return MSMGB_ERR_ARG;
    const double A = prm[0], xi = prm[1], P = prm[2], Q = prm[3], r0 = prm[4];
    const double csiv = 1.0 / ((double)ntab / std::sqrt(rmax));
    for (int i = 1; i <= ntab; ++i) {
        double t = (double)i * csiv;
        double r = t * t;
        double a = r / r0 - 1.0;
        double V = A * std::exp(-P * a);
        double rho = xi * xi * std::exp(-2.0 * Q * a);
        double fpotr = 2.0 * V * P * r / r0;
        double fpotb = 2.0 * Q * rho / r0;
        double v[5][3] = {
            {fpotr / A, 0.0, 0.0},
            {0.0, 2.0 * rho / xi, 2.0 * fpotb / xi},
            {2.0 * r * V * (1.0 - P * a) / r0, 0.0, 0.0},
            {0.0, -2.0 * a * rho, 2.0 * rho * (1.0 - 2.0 * Q * a) / r0},
            {2.0 * P * r * V * (P * r / r0 - 1.0) / (r0 * r0), 2.0 * Q * r * rho / (r0 * r0),
             2.0 * Q * rho * (2.0 * Q * r / r0 - 1.0) / (r0 * r0)}};
        for (int m = 0; m < 5; ++m)
            for (int k = 0; k < 3; ++k) d[(size_t)(m * 3 + k) * ntab + (i - 1)] = v[m][k];
    }
    return MSMGB_OK;
}
