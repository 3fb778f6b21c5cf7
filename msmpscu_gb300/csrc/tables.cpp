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
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

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

// Marinica EAM2, EAM3, EAM4 for W (EAM2/3/4_WW_Marinica_JPCM25_2013.F90): V a sum of 14-15
// cubic knots, rho of 4 knots frozen below RC = 2.002970124727 A, F = f1 sqrt(rho) + f2 rho^2.
// Literals without an exponent letter in those files are single precision and are written
// here as float literals: EAM2's knot radii, EAM3's knot radii and embedding coefficients,
// EAM4's pair knot radii.
struct MarSet {
    int nv;
    double a[15], r[15], b[4], rb[4], f[2];
};

const MarSet kMar[3] = {
    {15,
     {0.960851701343041e2, -0.184410923895214e3, 0.935784079613550e2, -0.798358265041677e1,
      0.747034092936229e1, -0.152756043708453e1, 0.125205932634393e1, 0.163082162159425e1,
      -0.141854775352260e1, -0.819936046256149e0, 0.198013514305908e1, -0.696430179520267e0,
      0.304546909722160e-1, -0.163131143161660e1, 0.138409896486177e1},
     {2.5648975f, 2.629795f, 2.6946925f, 2.8663175f, 2.973045f, 3.0797725f, 3.5164725f, 3.846445f,
      4.1764175f, 4.700845f, 4.8953f, 5.089755f, 5.3429525f, 5.401695f, 5.4604375f},
     {-0.420429107805055e1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.5f, 3.1f, 3.5f, 4.9f},
     {-5.946454472402710, -0.049477376935239}},
    {14,
     {0.335180090207171e3, -0.630187843239795e3, 0.351436490059390e3, -0.187104554936536e-1,
      0.599698179163370e-1, -0.210635074070024e-1, 0.258575483268791e-1, 0.389896994857220e-1,
      -0.139737073858817e-1, 0.184785876328131e-1, -0.505971175928021e0, -0.890738292956047e1,
      0.495992901621487e-1, 0.377639491131043e-1},
     {2.61f, 2.68f, 2.71816025391593f, 2.75852291093924f, 2.89242768139096f, 3.4015171088841f,
      3.67528316716263f, 4.24839261315764f, 4.63102917008654f, 4.82264509508677f, 5.02121483593414f,
      5.2828858486271f, 5.28302924730536f, 5.29092563021923f},
     {-0.420429107805055e-1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.5f, 3.1f, 3.5f, 4.9f},
     {-5.0732379057085f, -0.039263610952181f}},
    {15,
     {0.954071477542914e2, -0.181161004448916e3, 0.930215233132627e2, -0.108428907515182e2,
      0.112027468539573e2, -0.312459176640227e1, 0.123028140617302e1, 0.154767467307454e1,
      -0.128861387780439e1, -0.843327493551467e0, 0.214009882965042e1, -0.102898314532388e1,
      0.138163259601912e1, -0.360872433001551e1, 0.217655968740690e1},
     {2.5648975f, 2.629795f, 2.6946925f, 2.8663175f, 2.973045f, 3.0797725f, 3.5164725f, 3.846445f,
      4.1764175f, 4.700845f, 4.8953f, 5.089755f, 5.3429525f, 5.401695f, 5.4604375f},
     {-0.420429107805055e-1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.5, 3.1, 3.5, 4.9},
     {-5.553986589859130, -0.045691157657292}}};
const double kMarRC = 2.002970124727;

void cubic_knots(double rt, const double *a, const double *ri, int n, double *v, double *f)
{
    double p = 0.0, d = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = ri[i];
        double stp = (r - rt) >= 0.0 ? 1.0 : 0.0;
        p = p + a[i] * (r - rt) * (r - rt) * (r - rt) * stp;
        d = d + a[i] * (r - rt) * (r - rt) * stp;
    }
    *v = p;
    *f = 3.0 * d;
}

PairVal marinica(const MarSet &m, double r)
{
    PairVal o;
    double v, f;
    cubic_knots(r, m.a, m.r, m.nv, &v, &f);
    o.potr = 0.5 * v;            // NN_FuncPoly3 returns 0.5 V and -V'
    o.fpotr = f;
    if (r <= kMarRC) {           // density frozen inside RC
        cubic_knots(kMarRC, m.b, m.rb, 4, &o.potb, &o.fpotb);
        o.fpotb = 0.0;
    } else {
        cubic_knots(r, m.b, m.rb, 4, &o.potb, &o.fpotb);
    }
    return o;
}

void marinica_embed(const MarSet &m, double rho, double *f, double *df)
{
    if (rho <= 0.0) { *f = 0.0; *df = 0.0; return; }
    *f = m.f[0] * std::sqrt(rho) + m.f[1] * rho * rho;
    *df = 0.5 * m.f[0] / std::sqrt(rho) + 2.0 * m.f[1] * rho;
}

PairVal marinica2(double r) { return marinica(kMar[0], r); }
void marinica2_embed(double rho, double *f, double *df) { marinica_embed(kMar[0], rho, f, df); }

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

// The W-He library of the reference (EM_TB_WangJun_W-HE_2010, registered by
// EM_TB_ForceTable_WangJun_W_HE_2010.F90:68-121).  These three are evaluated in the reference's
// CGS units (cm, erg) exactly as written there and converted to Angstrom / eV on return.
const double kEVERG = 1.60219e-12;      // eV -> erg (MSM_Const.F90:83)
const double kBOHR = 5.291772108e-9;    // cm (MSM_Const.F90:99)
const double kPI = 3.141592654;         // CP_PI (MSM_Const.F90:56), as the reference states it

PairVal to_ev(double potr_erg, double fpotr_erg_cm)
{
    return PairVal{potr_erg / kEVERG, fpotr_erg_cm / kEVERG * 1e-8, 0.0, 0.0};
}

// Derlet, Nguyen-Manh, Dudarev W (FS form), FS_PM_WW.F90:7-204: V = sum_k v_k (rv_k - r)^3,
// rho = A^2 sum_k f_k (rf_k - r)^3 over the knots with r <= knot.  A is written without an
// exponent letter (:13), i.e. as a single-precision literal, so its value is that float.
PairVal derlet_ww(double r_a)
{
    static const double rv[9] = {4.2689e-8, 3.98568e-8, 3.70246e-8, 3.41924e-8, 3.13602e-8,
                                 2.8528e-8, 2.74110e-8, 2.604045e-8, 2.46699e-8};
    static const double v[9] = {-0.1036435865158945e24, -0.2912948318493851e24, -2.096765499656263e24,
                                19.1604545270101e24, -41.01619862085917e24, 46.05205617244703e24,
                                26.42203930654883e24, 15.35211507804088e24, 14.12806259323987e24};
    static const double rf[7] = {3.3216e-8, 3.165333333333333e-8, 3.009066666666667e-8, 2.8528e-8,
                                 2.7411e-8, 2.604045e-8, 2.46699e-8};
    static const double f[7] = {1.677334871575606e24, -1.673137509507131e24, -4.737051994974169e24,
                                7.870789420780674e24, -3.7924230525563378e20, 6.190816158916646e24,
                                -0.9565713891199151e24};
    const double A = (double)10.84238200368439f * kEVERG;
    const double r = r_a * 1e-8;
    double pv = 0.0, dv = 0.0, pb = 0.0, db = 0.0;
    for (int k = 0; k < 9; ++k)
        if (!(r > rv[k])) {
            const double t = rv[k] - r;
            pv += v[k] * kEVERG * t * t * t;
            dv += 3.0 * v[k] * kEVERG * t * t;
        }
    for (int k = 0; k < 7; ++k)
        if (!(r > rf[k])) {
            const double t = rf[k] - r;
            pb += f[k] * t * t * t;
            db += 3.0 * f[k] * t * t;
        }
    PairVal o = to_ev(0.5 * pv, dv);
    o.potb = pb * A * A / (kEVERG * kEVERG);          // eV^2
    o.fpotb = db * A * A / (kEVERG * kEVERG) * 1e-8;  // eV^2 / A
    return o;
}

// universal ZBL screened Coulomb pair, MD_CorePotent.F90:24-75 (CGS): POTR = V/2, FPOTR = -V'
void zbl_cgs(double z1, double z2, double r, double *potr, double *fpotr)
{
    const double ke2 = 9.0e9 * 1.60219e-19 * 1.60219e-19 * 1.0e7 * 1.0e2;
    const double as = 0.88534 * kBOHR / (std::pow(z1, 0.23) + std::pow(z2, 0.23));
    const double x = r / as, zz = z1 * z2 * ke2;
    const double e1 = std::exp(-3.1998 * x), e2 = std::exp(-0.94229 * x), e3 = std::exp(-0.4029 * x),
                 e4 = std::exp(-0.20162 * x);
    const double phi = zz * (0.18175 * e1 + 0.50986 * e2 + 0.28022 * e3 + 0.028171 * e4) / r;
    const double dphi = zz * (3.1998 * 0.18175 * e1 + 0.94229 * 0.50986 * e2 + 0.4029 * 0.28022 * e3 +
                              0.20162 * 0.028171 * e4) / as;
    *potr = 0.5 * phi;
    *fpotr = (phi + dphi) / r;
}

// He-He, ZBL_EXP6_HeHe.F90:7-86: ZBL below 1.0 A, a cubic bridge to 1.3 A, EXP6 beyond; no
// density.  The bridge's last two coefficients (:9-12) are written without an exponent letter,
// i.e. as single-precision literals, so they take their float values.
PairVal hehe_exp6(double r_a)
{
    static const double sc[4] = {3.5443059983603055e-11, -4.8619762395294636e-3, (double)200609.6243721997f,
                                 (double)-2069784026620.333f};
    const double r = r_a * 1e-8;
    double p, f;
    if (r < 1.0e-8) {
        zbl_cgs(2.0, 2.0, r, &p, &f);
    } else if (r < 1.3e-8) {
        p = (sc[0] + sc[1] * r + sc[2] * r * r + sc[3] * r * r * r) * 0.5;
        f = -(sc[1] + 2.0 * sc[2] * r + 3.0 * sc[3] * r * r);
    } else {
        const double ce = 0.000930644 * kEVERG, r0 = 0.29673e-7, alpha = 13.1;
        const double redx = r0 / r, ex = std::exp(alpha * (1.0 - 1.0 / redx));
        p = 0.5 * ce * (6.0 / (alpha - 6.0) * ex - (alpha / (alpha - 6.0)) * std::pow(redx, 6.0));
        f = ce * (6.0 / (alpha - 6.0) * ex * alpha / r0 -
                  (alpha / (alpha - 6.0)) * 6.0 * std::pow(redx, 5.0) * r0 / r / r);
    }
    return to_ev(p, f);
}

// He-W, ZBL_ABINTIO_He_W_930.F90:58-176: ZBL (SI constants) below 1.578 A, six cubic pieces in
// A / eV to 3.5 A, then an EXP6 form times a sine switch between 4.3 and 7.3 A.  The switch's
// derivative is taken as -cos(phase)/2 without the phase's own derivative (:147), and is kept so.
PairVal hew_zbl(double r_a)
{
    const double ep0 = 8.854187817e-12, qe = 1.60219e-19, z1 = 2.0, z2 = 74.0, a0 = 5.291772108e-11;
    static const double mid[7] = {1.57783601880074, 1.94810507446527, 2.10799896717072, 2.22277348041534,
                                  2.32289959788322, 3.05974050760269, 3.5};
    static const double cub[6][4] = {
        {-54.6920134504158, 147.764553002780, -106.604073601512, 23.3457856042901},
        {8.13894099222489, -6.77821270976276, 2.38825082778931, -0.378954410552979},
        {11.8316959842284, -9.92672851472125, 2.88240909576416, -0.299054384231567},
        {18.5956897803305, -18.0913941109865, 6.12169742584229, -0.719758272171021},
        {11.5965650160971, -9.38901671011024, 2.52039670944214, -0.223789215087891},
        {11.0095425643702, -9.03994004997097, 2.48033046722412, -0.227488279342651}};
    const double r = r_a * 1e-8, rr = r * 1.0e8;
    double p = 0.0, f = 0.0;
    if (r < mid[0] * 1.0e-8) {
        const double a = 0.88534 * a0 / (std::pow(z1, 0.23) + std::pow(z2, 0.23));
        const double x = r * 1.0e-2 / a;
        const double e1 = std::exp(-3.1998 * x), e2 = std::exp(-0.94229 * x), e3 = std::exp(-0.4029 * x),
                     e4 = std::exp(-0.20162 * x);
        const double faix = 0.18175 * e1 + 0.50986 * e2 + 0.28022 * e3 + 0.028171 * e4;
        const double dfaix = (0.18175 * e1 * (-3.1998) + 0.50986 * e2 * (-0.94229) + 0.28022 * e3 * (-0.4029) +
                              0.028171 * e4 * (-0.20162)) / a;
        p = 0.5 * (qe * z1 * z2 * faix / (4.0 * kPI * ep0 * r * 1.0e-2)) * kEVERG;
        f = -kEVERG * (qe * z1 * z2 / (4.0 * kPI * ep0) * (dfaix * r - faix * 1.0e2) / r / r);
    } else if (r < 3.5e-8) {
        int k = 0;
        while (k < 5 && !(r < mid[k + 1] * 1.0e-8)) ++k;
        const double *c = cub[k];
        p = kEVERG * 0.5 * (c[0] + c[1] * rr + c[2] * std::pow(rr, 2.0) + c[3] * std::pow(rr, 3.0));
        f = -kEVERG * (c[1] + 2.0 * c[2] * rr + 3.0 * c[3] * std::pow(rr, 2.0)) * 1.0e8;
    } else {
        const double cutrr = 5.8, cutorin = 1.5, ea = 0.0084600, eb = 9.6004204435, ec = 4.135;
        double fc, dfc;
        if (rr <= cutrr - cutorin) {
            fc = 1.0;
            dfc = 0.0;
        } else if (cutrr + cutorin <= rr) {
            fc = 0.0;
            dfc = 0.0;
        } else {
            const double ph = 3.141592654 * 0.5 * (rr - cutrr) / cutorin;
            dfc = -0.5 * std::cos(ph);
            fc = 0.5 * (1.0 - std::sin(ph));
        }
        const double zb = 6.0 / (eb - 6.0) * std::exp(eb * (1.0 - rr / ec));
        const double pm = ea * (zb - eb / (eb - 6.0) * std::pow(ec / rr, 6.0));
        double fp = -zb * eb / ec + eb / (eb - 6.0) * 6.0 * std::pow(ec / rr, 5.0) * ec / rr / rr;
        fp = ea * fp * fc + pm * dfc;
        p = kEVERG * 0.5 * (pm * fc);
        f = -kEVERG * fp * 1.0e8;
    }
    return to_ev(p, f);
}

// Ackland-Vitek Cu, Au and Cu-Au (EM_TB_Ackland_Vitek_PRB41_10324, FS form), evaluated in the
// reference's CGS units as written and converted on return.  Pair: Moliere screened Coulomb
// below R11, a fitted cubic to R21, then V/2 = sum_k AR_k (RCR_k - r)^3 over the knots above r;
// density: sum_k AT_k (RCT_k - r)^3 (Cu, Au) or the geometric mean sqrt(rho_Cu rho_Au) of the
// two (Cu-Au).  Single-precision literals of the source (Cu and Au knot coefficients and
// radii, Cu's screening length, the 0.3 of every Moliere derivative) are float literals here.
// The Cu-Au density derivative is written as 1.5 sum A A (X + Y) (X Y)^2 without the division
// by sqrt(P) (EM_TB_CuAu_Ackland_Vitek_PRB41_10324.F90:180-197); in CGS that is ~1e-24 of the
// true derivative, and it is kept so.
struct AVSet {
    double rrfit, ar[6], rcr[6], at[2], rct[2], r11, r21, as, z1, z2, ca[4];
};

AVSet av_cu()
{
    const double rr = 3.615e-08, e = kEVERG;
    const float a[6] = {61.73525861f, -108.1846780f, 57.00053948f, -12.88796578f, 39.163819010f, 0.0f};
    const float m[6] = {1.225f, 1.202f, 1.154f, 1.050f, 0.866f, 0.707f};
    AVSet s{};
    s.rrfit = rr;
    for (int k = 0; k < 6; ++k) {
        s.ar[k] = (double)a[k] * e * 0.5 / (rr * rr * rr);
        s.rcr[k] = (double)m[k] * rr;
    }
    s.at[0] = (double)10.03718305f * (e * e) / (rr * rr * rr);
    s.at[1] = (double)17.06363299f * (e * e) / (rr * rr * rr);
    s.rct[0] = (double)1.225f * rr;
    s.rct[1] = (double)0.990f * rr;
    s.r11 = 1.65e-8;
    s.r21 = 1.90e-8;
    s.as = (double)0.0738f * 1.0e-8;
    s.z1 = s.z2 = 29.0;
    s.ca[0] = 0.825015e-09; s.ca[1] = -0.130825; s.ca[2] = 0.696400e+07; s.ca[3] = -0.124069e+15;
    return s;
}

AVSet av_au()
{
    const double rr = 4.078e-08, e = kEVERG;
    const float a[6] = {29.059066f, -153.14779f, 148.17881f, -22.20508f, 72.71465f, 199.26269f};
    const float m[6] = {1.2247449f, 1.1547054f, 1.1180065f, 1.0000000f, 0.8660254f, 0.7071068f};
    AVSet s{};
    s.rrfit = rr;
    for (int k = 0; k < 6; ++k) {
        s.ar[k] = (double)a[k] * e * 0.5 / (rr * rr * rr);
        s.rcr[k] = (double)m[k] * rr;
    }
    s.at[0] = (double)21.930125f * (e * e) / (rr * rr * rr);
    s.at[1] = (double)284.99631f * (e * e) / (rr * rr * rr);
    s.rct[0] = (double)1.1180065f * rr;
    s.rct[1] = (double)0.8660254f * rr;
    s.r11 = 1.85e-8;
    s.r21 = 2.10e-8;
    s.as = 0.0752 * 1.0e-8;
    s.z1 = s.z2 = 79.0;
    s.ca[0] = 0.333482e-08; s.ca[1] = -0.476248; s.ca[2] = 0.228187e+08; s.ca[3] = -0.365939e+15;
    return s;
}

AVSet av_cuau()
{
    const double e = kEVERG;
    AVSet s{};
    const double a[3] = {-0.0855455166e24, 0.1928358800e24, 0.7593228600e24};
    const double rc[3] = {4.3098160e-08, 4.0474790e-08, 3.2979464e-08};
    for (int k = 0; k < 3; ++k) {
        s.ar[k] = a[k] * e * 0.5;
        s.rcr[k] = rc[k];
    }
    s.r11 = 1.85e-8;
    s.r21 = 2.05e-8;
    s.as = 0.0745 * 1.0e-8;
    s.z1 = 29.0;
    s.z2 = 79.0;
    s.ca[0] = 0.172724e-08; s.ca[1] = -0.253573; s.ca[2] = 0.124675e+08; s.ca[3] = -0.204896e+15;
    return s;
}

void av_pair_cgs(const AVSet &s, double r, double *potr, double *fpotr)
{
    if (r < s.r11) {
        const double zze2 = 9.0e9 * s.z1 * s.z2 * 1.6029e-19 * 1.6029e-19 * 1.0e9;
        const double be1 = std::exp(-0.3 * r / s.as), be2 = std::pow(be1, 4.0), be3 = std::pow(be2, 5.0);
        const double tp = zze2 * (0.35 * be1 + 0.55 * be2 + 0.1 * be3) / r;
        *potr = tp / 2.0;
        *fpotr = tp / r + zze2 * (0.35 * (double)0.3f * be1 + 0.55 * 1.2 * be2 + 0.1 * 6.0 * be3) / (r * s.as);
    } else if (r < s.r21) {
        *potr = (s.ca[0] + s.ca[1] * r + s.ca[2] * r * r + s.ca[3] * r * r * r) / 2.0;
        *fpotr = -(s.ca[1] + 2.0 * s.ca[2] * r + 3.0 * s.ca[3] * r * r);
    } else {
        double p = 0.0, f = 0.0;
        for (int k = 0; k < 6; ++k)
            if (r < s.rcr[k]) {
                p += s.ar[k] * std::pow(s.rcr[k] - r, 3.0);
                f += 6.0 * s.ar[k] * std::pow(s.rcr[k] - r, 2.0);
            }
        *potr = p;
        *fpotr = f;
    }
}

void av_rho_cgs(const AVSet &s, double r, double *potb, double *fpotb)
{
    *potb = 0.0;
    *fpotb = 0.0;
    for (int k = 0; k < 2; ++k)
        if (r > 0.0 && r < s.rct[k]) {
            *potb += s.at[k] * std::pow(s.rct[k] - r, 3.0);
            *fpotb += 3.0 * s.at[k] * std::pow(s.rct[k] - r, 2.0);
        }
}

PairVal ackland_vitek(int which, double r_a)
{
    const double r = r_a * 1e-8;
    const AVSet s = which == 0 ? av_cu() : which == 1 ? av_au() : av_cuau();
    double p, f, b = 0.0, db = 0.0;
    av_pair_cgs(s, r, &p, &f);
    if (which < 2) {
        av_rho_cgs(s, r, &b, &db);
    } else {
        const AVSet cu = av_cu(), au = av_au();
        const double x1 = cu.rct[0] - r, y1 = cu.rct[1] - r, x2 = au.rct[0] - r, y2 = au.rct[1] - r;
        double q = 0.0, dq = 0.0;
        if (r > 0.0 && r < au.rct[1]) {
            q = au.at[0] * cu.at[0] * std::pow(x2 * x1, 3.0) + au.at[0] * cu.at[1] * std::pow(x2 * y1, 3.0) +
                au.at[1] * cu.at[0] * std::pow(y2 * x1, 3.0) + au.at[1] * cu.at[1] * std::pow(y2 * y1, 3.0);
            dq = 1.5 * au.at[0] * cu.at[0] * (x2 + x1) * std::pow(x2 * x1, 2.0) +
                 1.5 * au.at[0] * cu.at[1] * (x2 + y1) * std::pow(x2 * y1, 2.0) +
                 1.5 * au.at[1] * cu.at[0] * (y2 + x1) * std::pow(y2 * x1, 2.0) +
                 1.5 * au.at[1] * cu.at[1] * (y2 + y1) * std::pow(y2 * y1, 2.0);
        } else if (r >= au.rct[1] && r < cu.rct[1]) {
            q = au.at[0] * cu.at[0] * std::pow(x2 * x1, 3.0) + au.at[0] * cu.at[1] * std::pow(x2 * y1, 3.0);
            dq = 1.5 * au.at[0] * cu.at[0] * (x2 + x1) * std::pow(x2 * x1, 2.0) +
                 1.5 * au.at[0] * cu.at[1] * (x2 + y1) * std::pow(x2 * y1, 2.0);
        } else if (r >= cu.rct[1] && r < cu.rct[0]) {
            q = au.at[0] * cu.at[0] * std::pow(x2 * x1, 3.0);
            dq = 1.5 * au.at[0] * cu.at[0] * (x2 + x1) * std::pow(x2 * x1, 2.0);
        }
        b = q > 0.0 ? std::sqrt(q) : 0.0;
        db = dq;
    }
    PairVal o = to_ev(p, f);
    o.potb = b / (kEVERG * kEVERG);
    o.fpotb = db / (kEVERG * kEVERG) * 1e-8;
    return o;
}

// Mendelev-Ackland Zr EAM (EAM_ZrZr_Mendelev_Phil_Mag_L87_2007.F90:18-150), in Angstrom / eV
// like the source: a screened Coulomb pair below 1 A, exp(cubic) to 2.3 A, then sums of
// (r_k - r)^n knots (n = 4..8); density knots at 5.6 A; F = -sqrt(rho) + sum_k c_k (rho - rho_k)^4.
// Single-precision literals of the source (the four screening weights and the knot radii
// 2.3, 5.6, 7.6) are float literals here.  H(x) = [x >= 0], H0(x) = [x > 0] (:172-192).
// F'(0) is -0.5/sqrt(0) = -inf in the first embedding row, as in the reference.
PairVal mendelev_zr(double r)
{
    auto H = [](double x) { return x >= 0.0 ? 1.0 : 0.0; };
    auto H0 = [](double x) { return x > 0.0 ? 1.0 : 0.0; };
    const double w[4] = {0.1818f, 0.5099f, 0.2802f, 0.02817f};
    const double b[4] = {3.3035595072498e+01, 9.7279503865046e+00, 4.1593878920967e+00, 2.0812424895674e+00};
    const double k23 = 2.3000f, k56 = 5.6f, k76 = 7.6f;
    const double kn[3] = {3.5, 6.0, k76};
    const double c[3][5] = {
        {-1.4261501929757e+01, 1.5850036758176e+01, -1.1325102264291e+01, -4.0971114831366e+00, 3.6739378016909e+00},
        {1.3066813393823e+00, -6.0542710718094e-01, 1.0055527194350e+00, -1.4918186777562e-01, 3.2773112059590e-02},
        {1.1433120304691e-02, -2.1982172508973e-02, -1.2542439692607e-02, 2.5062673874258e-02, -7.5442887837418e-03}};
    double v = 0.0, f = 0.0;
    if (H0(1.0 - r) > 0.0) {
        double s = 0.0, ds = 0.0;
        for (int k = 0; k < 4; ++k) {
            s += w[k] * std::exp(-b[k] * r);
            ds += (1.0 / r + b[k]) * w[k] * std::exp(-b[k] * r);
        }
        v += 2.3039613229091e+04 / r * s;
        f += 2.3039613229091e+04 / r * ds;
    }
    if (H(r - 1.0) * H0(k23 - r) > 0.0) {
        const double e = std::exp(1.2333392307614e+01 - 1.0847321969086e+01 * r + 4.5733524424508e+00 * r * r -
                                  8.5266291445935e-01 * r * r * r);
        v += e;
        f -= (-1.0847321969086e+01 + 9.1467048849017e+00 * r - 2.5579887433781e+00 * r * r) * e;
    }
    if (H(r - k23) > 0.0) {
        for (int g = 0; g < 3; ++g) {
            const double x = kn[g] - r;
            if (H(x) == 0.0) continue;
            double p = x * x * x;                       // x^3
            for (int n = 4; n <= 8; ++n) {
                f += c[g][n - 4] * n * p;
                p *= x;
                v += c[g][n - 4] * p;
            }
        }
    }
    PairVal o{0.5 * v, f, 0.0, 0.0};
    const double cr[5] = {7.7718711248373e-01, -4.8102928454986e-01, 1.4501312593993e-01, -2.1292226813959e-02,
                          1.2209217625670e-03};
    const double x = k56 - r;
    if (H(x) > 0.0) {
        double p = x * x * x;
        for (int n = 4; n <= 8; ++n) {
            o.fpotb += cr[n - 4] * n * p;
            p *= x;
            o.potb += cr[n - 4] * p;
        }
    }
    return o;
}

void mendelev_zr_embed(double rho, double *f, double *df)
{
    const double kr[5] = {60.0, 70.0, 80.0, 85.0, 90.0};
    const double kc[5] = {-1.9162462126235e-07, 4.6418727035037e-07, 6.6448294272955e-07, -2.0680252960229e-06,
                          1.1387131464983e-06};
    double a = -std::pow(rho, 0.5), d = -0.5 / std::pow(rho, 0.5);
    for (int k = 0; k < 5; ++k) {
        const double x = rho - kr[k];
        if (x < 0.0) continue;
        a += kc[k] * x * x * x * x;
        d += 4.0 * kc[k] * x * x * x;
    }
    *f = a;
    *df = d;
}

// Ackland-Wooding-Bacon Zr (EM_TB_AWB_Phil_Mag_A71_1995_553.F90, FS form), evaluated in CGS as
// written and converted on return: ZBL (Z = 40) below 1.2 A, exp(cubic in A) to 2.55 A, a cubic
// in cm to RCR7, then V = sum_k AR_k (RCR_k - r)^3 (7 knots) with POTR = V/2; density
// AT2 (RCT2 - r)^3 + AT1 (RCT1 - r)^3.  The knot coefficients and radii and B1..B4 are
// single-precision literals in the source.  Beyond RCR1 (pair) and RCT1 (density) the source
// assigns nothing, leaving the zero-initialised table entries (MD_TypeDef_ForceTable.F90:586).
PairVal awb_zr(double r_a)
{
    const double e = kEVERG, rr = 3.249e-08 * 1.414213562;     // RRFIT * CP_RSQ2
    const float ar[7] = {-58.480671f, 83.692945f, -20.958026f, -1.309533f, 65.726356f, 139.411255f, 443.442749f};
    const float mr[7] = {1.22f, 1.20f, 1.14f, 0.95f, 0.80f, 0.70f, 0.63f};
    const double r = r_a * 1e-8;
    double p = 0.0, f = 0.0;
    const double rcr7 = (double)mr[6] * rr;
    if (r < 1.20e-8) {
        zbl_cgs(40.0, 40.0, r, &p, &f);
    } else if (r <= 2.55e-8) {
        const double b1 = 13.4037f, b2 = -12.2190f, b3 = 5.0261f, b4 = -0.8435f;
        const double ra = r * 1e8;
        const double tp = e * std::exp(b1 + b2 * ra + b3 * ra * ra + b4 * ra * ra * ra);
        p = tp / 2.0;
        f = -(b2 + 2.0 * b3 * ra + 3.0 * b4 * ra * ra) * 1e8 * tp;
    } else if (r <= rcr7) {
        const double c3 = -19388949878932.86, c2 = 1706444.034874689, c1 = -5.0454065151782766e-002,
                     c0 = 5.0256487041006336e-010;
        p = (c0 + c1 * r + c2 * std::pow(r, 2.0) + c3 * std::pow(r, 3.0)) * 0.5;
        f = -(c1 + 2.0 * c2 * r + 3.0 * c3 * std::pow(r, 2.0));
    } else {
        for (int k = 0; k < 7; ++k) {
            const double rk = (double)mr[k] * rr, a = (double)ar[k] * e / (rr * rr * rr);
            if (r < rk) {
                p += a * std::pow(rk - r, 3.0);
                f += 3.0 * a * std::pow(rk - r, 2.0);
            }
        }
        p *= 0.5;
    }
    PairVal o = to_ev(p, f);
    const double rct1 = (double)1.22f * rr, rct2 = (double)1.05f * rr;
    const double at1 = (double)48.288836f * (e * e) / (rr * rr * rr), at2 = (double)-0.850556f * (e * e) / (rr * rr * rr);
    double b = 0.0, db = 0.0;
    if (r > 0.0 && r < rct2) {
        b = at2 * std::pow(rct2 - r, 3.0) + at1 * std::pow(rct1 - r, 3.0);
        db = 3.0 * at2 * std::pow(rct2 - r, 2.0) + 3.0 * at1 * std::pow(rct1 - r, 2.0);
    } else if (r >= rct2 && r < rct1) {
        b = at1 * std::pow(rct1 - r, 3.0);
        db = 3.0 * at1 * std::pow(rct1 - r, 2.0);
    }
    o.potb = b / (e * e);
    o.fpotb = db / (e * e) * 1e-8;
    return o;
}

// He-Ti of the reference's Ti-He library (LJ_He_Ti.F90:10-28, NN_HeTi_Interaction; no density),
// in CGS as written: V = pha0 ((r0/r)^4.35 - 3.211829 (r0/r)^1.4).  Both exponents are
// single-precision literals while the derivative's factors 4.35D0 and 1.4D0 are double, so
// -V' differs from the derivative of V in the eighth digit; kept so.
PairVal heti_lj(double r_a)
{
    const double pha0 = 0.02617 * kEVERG, r0 = 4.72879e-8;
    const double r = r_a * 1e-8, x = r0 / r;
    const double e1 = (double)4.35f, e2 = (double)1.4f;
    const double p = 0.5 * pha0 * (std::pow(x, e1) - 3.211829 * std::pow(x, e2));
    const double f = 0.5 * 2.0 * pha0 * (4.35 * std::pow(x, e1) / r - 3.211829 * 1.4 * std::pow(x, e2) / r);
    return to_ev(p, f);
}

// Bonny, Grigorev, Terentyev W-H-He EAM (EAM_WHeH_Bonny_JPCM26_2014), subtypes EAM1 and EAM2
// (EAM1_WHeH_Bonny_JPCM26_2014.F90).  W-W is Marinica EAM2 under a gauge transformation
// (:15-104); the other pairs are sums of cubic knots (NN_FuncPoly3,
// MD_Pot_EAM_Utilities.F90:48-85: POTR = V/2, FPOTR = -V').
PairVal poly3_pair(double r, const double *a, const double *ri, int n)
{
    double p = 0.0, d = 0.0;
    for (int i = 0; i < n; ++i)
        if (ri[i] - r >= 0.0) {
            p += a[i] * (ri[i] - r) * (ri[i] - r) * (ri[i] - r);
            d += a[i] * (ri[i] - r) * (ri[i] - r);
        }
    return PairVal{0.5 * p, 3.0 * d, 0.0, 0.0};
}

const double kBonC = 1.848055990, kBonS = 2.232322602e-1;

PairVal bonny_ww(double r)
{
    const PairVal m = marinica2(r);
    return PairVal{m.potr - kBonC * m.potb, m.fpotr - 2.0 * kBonC * m.fpotb, m.potb * kBonS, m.fpotb * kBonS};
}

void bonny_w_embed(double rho, double *f, double *df)
{
    const double is = 1.0 / kBonS, cos_ = kBonC * is;
    if (rho <= 1.359141225) {
        const double t = rho * is;
        double tf, tdf;
        marinica2_embed(t, &tf, &tdf);
        *f = tf + kBonC * t;
        *df = tdf * is + cos_;
    } else {
        const double a0 = -5.524855802, a1 = 2.317313103e-1, a2 = -3.665345949e-2, a3 = 8.989367404e-3;
        *f = a0 + rho * (a1 + rho * (a2 + rho * a3));
        *df = a1 + rho * (2.0 * a2 + 3.0 * a3 * rho);
    }
}

// EMBED_HH_Func2 through EMBED_FS_PLOY_Func (MD_Pot_EAM_Utilities.F90:332-368)
void bonny_h_embed(double rho, double *f, double *df)
{
    if (rho <= 0.0) { *f = 0.0; *df = 0.0; return; }
    const double a1 = -2.610066441e+01, a2 = 4.688963869e-01;
    *f = a1 * std::sqrt(rho) + a2 * rho * rho;
    *df = 0.5 * a1 / std::sqrt(rho) + 2.0 * a2 * rho;
}

// pair functions NN_*_Func1 (EAM1) and NN_*_Func2 (EAM2) for W-H, W-He, H-H, H-He, He-He
PairVal bonny_pair(int sub, int which, double r)
{
    static const double wh1a[2] = {1.375733214e+01, 1.296071475e-01}, wh1r[2] = {2.0, 3.0};
    static const double whe1a[3] = {2.100000000e+01, 8.565323293e-01, 2.750099819e-01}, whe1r[3] = {1.9, 2.2, 3.5};
    static const double hh1a[2] = {4.862785907e-01, 1.018797872e-01}, hh1r[2] = {2.0, 3.0};
    static const double hhe1a[3] = {1.500000000e+01, 2.563700119e-01, -4.489510592e-02}, hhe1r[3] = {1.8, 2.0, 3.0};
    static const double hehe1a[2] = {2.106615791e+00, -2.217639348e-01}, hehe1r[2] = {2.0, 3.0};
    static const double wh2a[3] = {4.424459079e+01, -4.993477782e+00, 1.461712984e+00},
                        wh2r[3] = {2.0, 2.6475, 3.295};
    static const double whe2a[4] = {0.0, 1.400000000e+01, -3.712116187e+00, 3.105031456e-01},
                        whe2r[4] = {1.9, 2.0, 2.2, 3.5};
    static const double hh2a[4] = {4.000000000e+01, 2.315124670e-01, -2.000000000e-01, 5.180584543e-02},
                        hh2r[4] = {1.6, 2.0, 2.2, 3.0};
    static const double hhe2a[3] = {3.256370012e+00, -4.000000000e-01, -4.489510592e-02}, hhe2r[3] = {2.0, 2.5, 3.0};
    static const double hehe2a[4] = {2.000000000e+01, 1.051327582e+00, -4.000000000e+00, 3.203322671e-02},
                        hehe2r[4] = {1.8, 2.0, 2.1, 3.0};
    switch (which * 2 + (sub == 2)) {
    case 0: return poly3_pair(r, wh1a, wh1r, 2);
    case 1: return poly3_pair(r, wh2a, wh2r, 3);
    case 2: return poly3_pair(r, whe1a, whe1r, 3);
    case 3: return poly3_pair(r, whe2a, whe2r, 4);
    case 4: return poly3_pair(r, hh1a, hh1r, 2);
    case 5: return poly3_pair(r, hh2a, hh2r, 4);
    case 6: return poly3_pair(r, hhe1a, hhe1r, 3);
    case 7: return poly3_pair(r, hhe2a, hhe2r, 3);
    case 8: return poly3_pair(r, hehe1a, hehe1r, 2);
    default: return poly3_pair(r, hehe2a, hehe2r, 4);
    }
}

}  // namespace

extern "C" int msmgb_create_forcetable(int pot, const double *prm, double rmax, int ntab,
                                       int nembd, double rhoscal, double *potr, double *fpotr,
                                       double *potb, double *fpotb, double *fembd,
                                       double *dfembd, double *rhod)
{
    if (ntab < 2 || rmax <= 0.0 || !potr || !fpotr || !potb || !fpotb) return MSMGB_ERR_ARG;
    if (pot == MSMGB_POT_CR && !prm) return MSMGB_ERR_ARG;
    if (pot < MSMGB_POT_CR || pot > MSMGB_POT_HETI_LJ) return MSMGB_ERR_ARG;
    const double csi = (double)ntab / std::sqrt(rmax);
    const double csiv = 1.0 / csi;
    double rhomx = -1.0;
    for (int i = 1; i <= ntab; ++i) {
        double t = (double)i * csiv;
        double r = t * t;
        PairVal v;
        switch (pot) {
        case MSMGB_POT_CR: v = cleri_rosato(r, prm); break;
        case MSMGB_POT_MARINICA2: v = marinica2(r); break;
        case MSMGB_POT_MARINICA3: v = marinica(kMar[1], r); break;
        case MSMGB_POT_MARINICA4: v = marinica(kMar[2], r); break;
        case MSMGB_POT_AV_CU: v = ackland_vitek(0, r); break;
        case MSMGB_POT_AV_AU: v = ackland_vitek(1, r); break;
        case MSMGB_POT_AV_CUAU: v = ackland_vitek(2, r); break;
        case MSMGB_POT_MENDELEV_ZR: v = mendelev_zr(r); break;
        case MSMGB_POT_AWB_ZR: v = awb_zr(r); break;
        case MSMGB_POT_HETI_LJ: v = heti_lj(r); break;
        case MSMGB_POT_ACKLAND_WW: v = ackland_ww(r); break;
        case MSMGB_POT_DERLET_WW: v = derlet_ww(r); break;
        case MSMGB_POT_HEHE_EXP6: v = hehe_exp6(r); break;
        default: v = hew_zbl(r); break;
        }
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
            if (pot == MSMGB_POT_MARINICA2 || pot == MSMGB_POT_MARINICA3 || pot == MSMGB_POT_MARINICA4) {
                const int set = pot == MSMGB_POT_MARINICA2 ? 0 : pot == MSMGB_POT_MARINICA3 ? 1 : 2;
                marinica_embed(kMar[set], rho, &fembd[i - 1], &dfembd[i - 1]);
            } else if (pot == MSMGB_POT_MENDELEV_ZR) {
                mendelev_zr_embed(rho, &fembd[i - 1], &dfembd[i - 1]);
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

// ---- tabulated EAM potentials in setfl layout -------------------------------------------
// Register_ForceTableProc_Setfl (Filedatas_Func_Setfl.F90:499-541) with the reader
// get_filedatas_setfl (:119-253): three comment lines; "NE el1 el2 ..."; "Nrho drho Nr dr
// cutoff"; per element a line "Z mass a lattice", Nrho values of F(rho) and Nr values of
// rho(r); then r*phi(r) for every pair I >= J.  The r grid is R_i = i cutoff/Nr, the rho grid
// i drho.  A leading "INF" / "NAN" token stands for the r = 0 value, which takes the next one.
// Interpolation: the reference uses SLATEC DBINT4/DBVALU with IBCL = IBCR = 2, FBCL = FBCR
// = 0 and KNTOPT = 1 (:25-34, 256-276), i.e. the natural cubic spline through the data.
namespace {

struct Setfl {
    int ne = 0, nrho = 0, nr = 0;
    double drho = 0.0, dr = 0.0, cutoff = 0.0;
    std::vector<double> mass;
    std::vector<std::vector<double>> frho, rhor;   // [element][point]
    std::vector<std::vector<double>> rphi;         // [I*(I+1)/2 + J], J <= I
};

bool next_token(FILE *f, std::string &t)
{
    t.clear();
    int c;
    while ((c = fgetc(f)) != EOF && (c == ' ' || c == '\t' || c == '\n' || c == '\r')) {}
    if (c == EOF) return false;
    do { t.push_back((char)c); } while ((c = fgetc(f)) != EOF && c != ' ' && c != '\t' && c != '\n' && c != '\r');
    return true;
}

bool read_block(FILE *f, int n, std::vector<double> &v)
{
    v.assign((size_t)n, 0.0);
    std::string t;
    bool first_special = false;
    for (int i = 0; i < n; ++i) {
        if (!next_token(f, t)) return false;
        if (i == 0 && (t == "INF" || t == "inf" || t == "NAN" || t == "nan")) {
            first_special = true;
            continue;
        }
        char *end = nullptr;
        v[(size_t)i] = strtod(t.c_str(), &end);
        if (end == t.c_str()) return false;
    }
    if (first_special) v[0] = n > 1 ? v[1] : 0.0;
    return true;
}

int read_setfl(const char *path, Setfl &s)
{
    FILE *f = fopen(path, "r");
    if (!f) return MSMGB_ERR_ARG;
    char line[4096];
    int rc = MSMGB_ERR_ARG;
    for (int k = 0; k < 3; ++k)
        if (!fgets(line, sizeof(line), f)) goto done;
    if (!fgets(line, sizeof(line), f) || sscanf(line, "%d", &s.ne) != 1 || s.ne < 1 || s.ne > 4) goto done;
    if (!fgets(line, sizeof(line), f) ||
        sscanf(line, "%d %lf %d %lf %lf", &s.nrho, &s.drho, &s.nr, &s.dr, &s.cutoff) != 5 || s.nrho < 3 ||
        s.nr < 3 || s.drho <= 0.0 || s.cutoff <= 0.0)
        goto done;
    s.mass.assign((size_t)s.ne, 0.0);
    s.frho.resize((size_t)s.ne);
    s.rhor.resize((size_t)s.ne);
    for (int e = 0; e < s.ne; ++e) {
        std::string t;
        if (!next_token(f, t)) goto done;                     // atomic number
        if (!next_token(f, t)) goto done;
        s.mass[(size_t)e] = strtod(t.c_str(), nullptr);
        if (!next_token(f, t) || !next_token(f, t)) goto done;   // lattice constant, structure
        if (!read_block(f, s.nrho, s.frho[(size_t)e]) || !read_block(f, s.nr, s.rhor[(size_t)e])) goto done;
    }
    s.rphi.resize((size_t)(s.ne * (s.ne + 1) / 2));
    for (int i = 0; i < s.ne; ++i)
        for (int j = 0; j <= i; ++j)
            if (!read_block(f, s.nr, s.rphi[(size_t)(i * (i + 1) / 2 + j)])) goto done;
    rc = MSMGB_OK;
done:
    fclose(f);
    return rc;
}

// natural cubic spline on x_i = i h: second derivatives (Thomas algorithm)
std::vector<double> spline_m(const std::vector<double> &y, double h)
{
    const size_t n = y.size();
    std::vector<double> m(n, 0.0), cp(n, 0.0);
    const double s = 6.0 / (h * h);
    for (size_t i = 1; i + 1 < n; ++i) {
        const double den = 4.0 - cp[i - 1];
        cp[i] = 1.0 / den;
        m[i] = (s * (y[i + 1] - 2.0 * y[i] + y[i - 1]) - m[i - 1]) / den;
    }
    m[n - 1] = 0.0;
    for (size_t i = n - 2; i >= 1; --i) m[i] -= cp[i] * m[i + 1];
    return m;
}

double spline_at(const std::vector<double> &y, const std::vector<double> &m, double h, double x, double *dy)
{
    const int n = (int)y.size();
    int k = (int)std::floor(x / h);
    if (k < 0) k = 0;
    if (k > n - 2) k = n - 2;
    const double b = (x - k * h) / h, a = 1.0 - b;
    if (dy)
        *dy = (y[(size_t)k + 1] - y[(size_t)k]) / h +
              h * ((1.0 - 3.0 * a * a) * m[(size_t)k] + (3.0 * b * b - 1.0) * m[(size_t)k + 1]) / 6.0;
    return a * y[(size_t)k] + b * y[(size_t)k + 1] +
           ((a * a * a - a) * m[(size_t)k] + (b * b * b - b) * m[(size_t)k + 1]) * (h * h / 6.0);
}

}  // namespace

extern "C" int msmgb_setfl_info(const char *path, int *nelem, int *nrho, int *nr, double *cutoff)
{
    if (!path) return MSMGB_ERR_ARG;
    Setfl s;
    int rc = read_setfl(path, s);
    if (rc) return rc;
    if (nelem) *nelem = s.ne;
    if (nrho) *nrho = s.nrho;
    if (nr) *nr = s.nr;
    if (cutoff) *cutoff = s.cutoff;
    return MSMGB_OK;
}

extern "C" int msmgb_setfl_tables(const char *path, int ntab, double *potr, double *fpotr, double *potb,
                                  double *fpotb, double *fembd, double *dfembd, int *kpair, int *kembd,
                                  double *rhod, double *masses)
{
    if (!path || ntab < 2 || !potr || !fpotr || !potb || !fpotb || !fembd || !dfembd || !kpair || !kembd)
        return MSMGB_ERR_ARG;
    Setfl s;
    int rc = read_setfl(path, s);
    if (rc) return rc;
    const int ne = s.ne, nk = ne * ne;
    const double dr = s.cutoff / s.nr;                 // R(I) = (I-1) cutoff/Nr
    const double rimax = (s.nr - 1) * dr, fimax = (s.nrho - 1) * s.drho;
    std::vector<std::vector<double>> mr((size_t)ne), mf((size_t)ne), mp(s.rphi.size());
    std::vector<int> fzero((size_t)ne, 1);
    for (int e = 0; e < ne; ++e) {
        mr[(size_t)e] = spline_m(s.rhor[(size_t)e], dr);
        mf[(size_t)e] = spline_m(s.frho[(size_t)e], s.drho);
        for (double v : s.frho[(size_t)e])
            if (v != 0.0) fzero[(size_t)e] = 0;
    }
    for (size_t q = 0; q < s.rphi.size(); ++q) mp[q] = spline_m(s.rphi[q], dr);
    const double csiv = std::sqrt(s.cutoff) / ntab;
    // table (I, J), 1-based id (I-1)*NE + J: pair phi_{max(I,J),min(I,J)}; density of a J atom
    // at an I atom (zero when element I has no embedding energy)
    for (int I = 0; I < ne; ++I)
        for (int J = 0; J < ne; ++J) {
            const int k = I * ne + J;
            const int a = I > J ? I : J, b = I > J ? J : I;
            const std::vector<double> &yp = s.rphi[(size_t)(a * (a + 1) / 2 + b)];
            const std::vector<double> &mpk = mp[(size_t)(a * (a + 1) / 2 + b)];
            for (int i = 1; i <= ntab; ++i) {
                const double t = i * csiv, r = t * t;
                double f = 0.0, df = 0.0, rho = 0.0, drh = 0.0;
                if (r <= rimax) {
                    f = spline_at(yp, mpk, dr, r, &df);
                    if (!fzero[(size_t)I]) rho = spline_at(s.rhor[(size_t)J], mr[(size_t)J], dr, r, &drh);
                }
                const double phi = f / r, dphi = (df - phi) / r;
                const size_t o = (size_t)(i - 1) * nk + k;  // (NKIND, NTAB) column-major
                potr[o] = 0.5 * phi * r;
                fpotr[o] = -dphi * r;
                potb[o] = rho;
                fpotb[o] = -drh;
            }
            kpair[J * ne + I] = k + 1;                      // KPAIR(I,J), column-major
        }
    for (int e = 0; e < ne; ++e) {
        kembd[e] = e + 1;
        for (int i = 1; i <= s.nrho; ++i) {
            const double rho = (i - 1) * s.drho;
            double d = 0.0, f;
            if (rho <= fimax) f = spline_at(s.frho[(size_t)e], mf[(size_t)e], s.drho, rho, &d);
            else f = spline_at(s.frho[(size_t)e], mf[(size_t)e], s.drho, fimax, nullptr);
            const size_t o = (size_t)(i - 1) * ne + e;      // (NKIND1, NEMBD) column-major
            fembd[o] = f;
            dfembd[o] = d;
        }
    }
    if (rhod) *rhod = s.drho;
    if (masses)
        for (int e = 0; e < ne; ++e) masses[e] = s.mass[(size_t)e];
    return MSMGB_OK;
}

// ---- tabulated EAM potentials in lspt layout ----------------------------------------------
// Register_ForceTableProc_SPT (Filedatas_Func_Lspt.F90:560-604) with the reader
// get_filedatas_lspt (:118-301).  The control file, read line by line with comment lines
// ('!') and blank lines skipped (GETINPUTSTRLINE.F): a line starting "&LSPT"; a line whose
// first number is the element count NE; a line of NE quoted element symbols; per element a
// line quoting its F(rho) file and one quoting its rho(r) file ("NA" = none); then for
// I = 1..NE a line quoting I pair files V(r) of element I with elements 1..I.  Quoted means
// between a pair of " or ' (EXSUBSTR.F).  Data files (".spt") hold '#' comment lines, then
// "x f(x)" lines; their paths are relative to the control file's folder.
// The reference opens the FIRST file named on each pair line for every pair of that line
// (:263, SUBSTR(1) inside the loop over J); msmgb_lspt_tables does the same unless it is
// given MSMGB_LSPT_EACH_VR_FILE.
// Evaluation (Vr_Spline :340-385, Rhor_Spline :388-443, Frho_Spline :446-500): natural cubic
// spline through the data (DBINT4 with IBCL = IBCR = 2, FBCL = FBCR = 0, KNTOPT = 1, :24-34);
// below the first x the value at the first x with zero derivative; above the last x zero for
// V(r) and rho(r), and F(x_last) with zero derivative for F(rho).  Tables take POTR = 0.5 V r,
// FPOTR = -V' r, POTB = rho, FPOTB = -rho' (NN_Spline, RHO_Spline :503-537).  The density at
// a host element without an F(rho) file is zero (the integer flag test at :406 read as "the
// host has an F(rho) file"; no force or energy depends on it).
// RMAX = the largest x of the pair files read (:291), RHOMX = the largest x of the F(rho) files
// (:290), RHOD = RHOMX / NEMBD: the NIST table generator restores the reader's RHOMX after
// building the pair tables (Generate_NIST_ForceTalbe, NIST_ForceTable.F90:379-413), so the
// RHOSCAL * max POTB rule of other libraries does not apply (RHOD = 1 when no F(rho) file).
namespace {

struct Spt {
    bool na = true;
    std::vector<double> x, y, m;
};

struct Lspt {
    int ne = 0;
    std::vector<Spt> frho, rhor;
    std::vector<Spt> vr;        // [I*(I+1)/2 + J], J <= I
    double rmax = 0.0, rhomax = 0.0;
};

// one input line as GETINPUTSTRLINE returns it: printable characters only, left-adjusted;
// false at end of file
bool ctl_line(FILE *f, const char *skip, std::string &s)
{
    char buf[4096];
    while (fgets(buf, sizeof(buf), f)) {
        s.clear();
        for (const char *p = buf; *p; ++p)
            if ((unsigned char)*p >= 20 && (unsigned char)*p <= 126) s.push_back(*p);
        size_t b = s.find_first_not_of(' ');
        if (b == std::string::npos) continue;
        s.erase(0, b);
        if (strchr(skip, s[0])) continue;
        return true;
    }
    return false;
}

std::vector<std::string> quoted(const std::string &s)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        if (s[i] == '"' || s[i] == '\'') {
            size_t e = s.find(s[i], i + 1);
            if (e == std::string::npos) break;
            out.push_back(s.substr(i + 1, e - i - 1));
            i = e + 1;
        } else {
            ++i;
        }
    }
    return out;
}

std::string trim(const std::string &s)
{
    size_t b = s.find_first_not_of(' '), e = s.find_last_not_of(' ');
    return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
}

bool is_na(const std::string &name)
{
    std::string t = trim(name);
    return t.size() == 2 && toupper((unsigned char)t[0]) == 'N' && toupper((unsigned char)t[1]) == 'A';
}

// natural cubic spline through (x_i, y_i), x strictly increasing: second derivatives
void spline_nu(Spt &s)
{
    const size_t n = s.x.size();
    s.m.assign(n, 0.0);
    if (n < 3) return;
    std::vector<double> c(n, 0.0);
    for (size_t i = 1; i + 1 < n; ++i) {
        const double h0 = s.x[i] - s.x[i - 1], h1 = s.x[i + 1] - s.x[i];
        const double rhs = 6.0 * ((s.y[i + 1] - s.y[i]) / h1 - (s.y[i] - s.y[i - 1]) / h0);
        const double den = 2.0 * (h0 + h1) - h0 * c[i - 1];
        c[i] = h1 / den;
        s.m[i] = (rhs - h0 * s.m[i - 1]) / den;
    }
    for (size_t i = n - 2; i >= 1; --i) s.m[i] -= c[i] * s.m[i + 1];
}

double spline_nu_at(const Spt &s, double t, double *dy)
{
    const size_t n = s.x.size();
    size_t lo = 0, hi = n - 1;                   // x[lo] <= t < x[hi]
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        if (s.x[mid] <= t) lo = mid; else hi = mid;
    }
    const double h = s.x[hi] - s.x[lo], b = (t - s.x[lo]) / h, a = 1.0 - b;
    if (dy)
        *dy = (s.y[hi] - s.y[lo]) / h + h * ((1.0 - 3.0 * a * a) * s.m[lo] + (3.0 * b * b - 1.0) * s.m[hi]) / 6.0;
    return a * s.y[lo] + b * s.y[hi] + ((a * a * a - a) * s.m[lo] + (b * b * b - b) * s.m[hi]) * (h * h / 6.0);
}

// value and derivative with the reader's range rules; above_keep: F(rho) keeps its last value
double spt_eval(const Spt &s, double t, bool above_keep, double *dy)
{
    *dy = 0.0;
    if (s.na) return 0.0;
    if (t < s.x.front()) return spline_nu_at(s, s.x.front(), nullptr);
    if (t <= s.x.back()) return spline_nu_at(s, t, dy);
    return above_keep ? spline_nu_at(s, s.x.back(), nullptr) : 0.0;
}

int read_spt(const std::string &path, Spt &s)
{
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return MSMGB_ERR_ARG;
    std::string line;
    int rc = MSMGB_OK;
    s.x.clear();
    s.y.clear();
    while (ctl_line(f, "#", line)) {
        char *e1 = nullptr, *e2 = nullptr;
        const double x = strtod(line.c_str(), &e1);
        const double y = strtod(e1, &e2);
        if (e1 == line.c_str() || e2 == e1) { rc = MSMGB_ERR_ARG; break; }
        if (!s.x.empty() && !(x > s.x.back())) { rc = MSMGB_ERR_ARG; break; }
        s.x.push_back(x);
        s.y.push_back(y);
    }
    fclose(f);
    if (rc == MSMGB_OK && s.x.size() < 2) rc = MSMGB_ERR_ARG;
    if (rc == MSMGB_OK) {
        s.na = false;
        spline_nu(s);
    }
    return rc;
}

int read_lspt(const char *path, int flags, Lspt &L)
{
    FILE *f = fopen(path, "r");
    if (!f) return MSMGB_ERR_ARG;
    std::string dir(path);
    const size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
    std::string s;
    int rc = MSMGB_ERR_ARG;
    std::vector<std::string> q;
    if (!ctl_line(f, "!", s)) goto done;
    {
        std::string kw = s.substr(0, s.find(' '));
        for (char &c : kw) c = (char)toupper((unsigned char)c);
        if (kw != "&LSPT") goto done;
    }
    if (!ctl_line(f, "!", s)) goto done;
    {
        size_t i = s.find_first_of("0123456789");
        if (i == std::string::npos) goto done;
        L.ne = atoi(s.c_str() + i);
        if (L.ne < 1 || L.ne > 4) goto done;
    }
    if (!ctl_line(f, "!", s) || (int)quoted(s).size() != L.ne) goto done;
    L.frho.resize((size_t)L.ne);
    L.rhor.resize((size_t)L.ne);
    L.vr.resize((size_t)(L.ne * (L.ne + 1) / 2));
    for (int e = 0; e < L.ne; ++e)
        for (int w = 0; w < 2; ++w) {
            if (!ctl_line(f, "!", s) || (q = quoted(s)).empty()) goto done;
            Spt &t = w == 0 ? L.frho[(size_t)e] : L.rhor[(size_t)e];
            if (is_na(q[0])) continue;
            if (read_spt(dir + trim(q[0]), t) != MSMGB_OK) goto done;
            if (w == 0 && t.x.back() > L.rhomax) L.rhomax = t.x.back();
        }
    for (int i = 0; i < L.ne; ++i) {
        if (!ctl_line(f, "!", s) || (int)(q = quoted(s)).size() != i + 1) goto done;
        for (int j = 0; j <= i; ++j) {
            Spt &t = L.vr[(size_t)(i * (i + 1) / 2 + j)];
            const std::string &name = (flags & MSMGB_LSPT_EACH_VR_FILE) ? q[(size_t)j] : q[0];
            if (read_spt(dir + trim(name), t) != MSMGB_OK) goto done;
            if (t.x.back() > L.rmax) L.rmax = t.x.back();
        }
    }
    rc = MSMGB_OK;
done:
    fclose(f);
    return rc;
}

}  // namespace

extern "C" int msmgb_lspt_info(const char *path, int flags, int *nelem, double *rmax, double *rhomax)
{
    if (!path) return MSMGB_ERR_ARG;
    Lspt L;
    int rc = read_lspt(path, flags, L);
    if (rc) return rc;
    if (nelem) *nelem = L.ne;
    if (rmax) *rmax = L.rmax;
    if (rhomax) *rhomax = L.rhomax;
    return MSMGB_OK;
}

extern "C" int msmgb_lspt_tables(const char *path, int flags, int ntab, int nembd, double rmax,
                                 double *potr, double *fpotr, double *potb, double *fpotb,
                                 double *fembd, double *dfembd, int *kpair, int *kembd, double *rhod)
{
    if (!path || ntab < 2 || nembd < 2 || !potr || !fpotr || !potb || !fpotb || !fembd || !dfembd || !kpair ||
        !kembd)
        return MSMGB_ERR_ARG;
    Lspt L;
    int rc = read_lspt(path, flags, L);
    if (rc) return rc;
    const int ne = L.ne, nk = ne * ne;
    if (!(rmax > 0.0)) rmax = L.rmax;
    const double csiv = std::sqrt(rmax) / ntab;
    // table (I, J), 1-based id (I-1)*NE + J (Notify_func :327-337): pair V of elements
    // max(I,J), min(I,J); density of element J at an element-I host
    for (int I = 0; I < ne; ++I)
        for (int J = 0; J < ne; ++J) {
            const int k = I * ne + J;
            const int a = I > J ? I : J, b = I > J ? J : I;
            const Spt &v = L.vr[(size_t)(a * (a + 1) / 2 + b)];
            const bool no_density = L.frho[(size_t)I].na;
            for (int i = 1; i <= ntab; ++i) {
                const double t = i * csiv, r = t * t;
                double dv = 0.0, drh = 0.0;
                const double vv = spt_eval(v, r, false, &dv);
                const double rho = no_density ? 0.0 : spt_eval(L.rhor[(size_t)J], r, false, &drh);
                const size_t o = (size_t)(i - 1) * nk + k;  // (NKIND, NTAB) column-major
                potr[o] = 0.5 * vv * r;
                fpotr[o] = -dv * r;
                potb[o] = rho;
                fpotb[o] = -drh;
            }
            kpair[J * ne + I] = k + 1;                      // KPAIR(I,J), column-major
        }
    const double d = L.rhomax > 0.0 ? L.rhomax / nembd : 1.0;
    for (int e = 0; e < ne; ++e) {
        kembd[e] = e + 1;
        for (int i = 1; i <= nembd; ++i) {
            double df = 0.0;
            const double f = spt_eval(L.frho[(size_t)e], (i - 1) * d, true, &df);
            const size_t o = (size_t)(i - 1) * ne + e;      // (NKIND1, NEMBD) column-major
            fembd[o] = f;
            dfembd[o] = df;
        }
    }
    if (rhod) *rhod = d;
    return MSMGB_OK;
}

// Register_Interaction_Table of EAM_ForceTable_Bonny_JPCM26_2014.F90 (:17-121): tables in the
// order the reference registers them, (source, target) = (W,W) (H,W) (He,W) (W,H) (H,H) (He,H)
// (W,He) (H,He) (He,He), plus a zero table #10 for EAM2.  The target is the host
// (Create_Interaction_ForceTable, MD_TypeDef_ForceTable.F90:1168-1178), so with groups
// W = 1, H = 2, He = 3 the host-I / neighbour-J table is KPAIR(I,J) = (I-1)*3 + J.
extern "C" int msmgb_bonny_wheh_tables(int subtype, double rmax, int ntab, int nembd, double rhoscal,
                                       double *potr, double *fpotr, double *potb, double *fpotb,
                                       double *fembd, double *dfembd, int *kpair, int *kembd, int *nkind,
                                       double *rhod)
{
    if ((subtype != 1 && subtype != 2) || rmax <= 0.0 || ntab < 2 || nembd < 2 || !potr || !fpotr || !potb ||
        !fpotb || !fembd || !dfembd || !kpair || !kembd)
        return MSMGB_ERR_ARG;
    if (!(rhoscal > 0.0)) rhoscal = 20.0;
    const int nk = subtype == 2 ? 10 : 9;
    // pair function per table: -1 W-W, else bonny_pair index (0 WH, 1 WHe, 2 HH, 3 HHe, 4 HeHe)
    static const int pairfn[10] = {-1, 0, 1, 0, 2, 3, 1, 3, 4, -2};
    const double csiv = std::sqrt(rmax) / ntab;
    double rhomx = 0.0;
    for (int k = 0; k < nk; ++k)
        for (int i = 1; i <= ntab; ++i) {
            const double t = i * csiv, r = t * t;
            PairVal v{0.0, 0.0, 0.0, 0.0};
            if (pairfn[k] == -1) {
                v = bonny_ww(r);
            } else if (pairfn[k] >= 0) {
                v = bonny_pair(subtype, pairfn[k], r);
                if (subtype == 2 && k == 3) {                // (W,H): the W density at an H host
                    const PairVal w = bonny_ww(r);
                    v.potb = w.potb;
                    v.fpotb = w.fpotb;
                }
            }
            const size_t o = (size_t)(i - 1) * nk + k;
            potr[o] = v.potr * r;
            fpotr[o] = v.fpotr * r;
            potb[o] = v.potb;
            fpotb[o] = v.fpotb;
            if (rhomx < v.potb * rhoscal) rhomx = v.potb * rhoscal;
        }
    const double d = rhomx / nembd;
    for (int i = 1; i <= nembd; ++i) {
        const double rho = (i - 1) * d;
        double f = 0.0, df = 0.0;
        bonny_w_embed(rho, &f, &df);
        fembd[(size_t)(i - 1) * 3 + 0] = f;
        dfembd[(size_t)(i - 1) * 3 + 0] = df;
        f = df = 0.0;
        if (subtype == 2) bonny_h_embed(rho, &f, &df);
        fembd[(size_t)(i - 1) * 3 + 1] = f;
        dfembd[(size_t)(i - 1) * 3 + 1] = df;
        fembd[(size_t)(i - 1) * 3 + 2] = 0.0;
        dfembd[(size_t)(i - 1) * 3 + 2] = 0.0;
    }
    for (int I = 0; I < 3; ++I) {
        kembd[I] = I + 1;
        for (int J = 0; J < 3; ++J) kpair[J * 3 + I] = I * 3 + J + 1;   // column-major
    }
    if (nkind) *nkind = nk;
    if (rhod) *rhod = d;
    return MSMGB_OK;
}

// ---- Moldy potential files ------------------------------------------------------------------
// Register_ForceTableProc_Moldy with the reader get_filedatas_moldy (Filedatas_Func_Moldy.F90:
// 27-77, 116-131): line 1 the element symbol; then four lines of numbers (pair coefficients
// a_k, pair knots r_k, density coefficients A_k, density knots R_k) and a line of constants
// whose first is the lattice constant a0; numbers are the tokens between blanks, commas,
// brackets and '=' (EXNUMB.F).  Knots scale by a0, a_k by a0^-3, A_k by a0^-6.  Pair
// V = sum a_k (r_k - r)^3 (NN_FuncPoly3: POTR = V/2, FPOTR = -V'), density
// rho = sum A_k (R_k - r)^3 (RHO_FuncPoly3), embedding F = -sqrt(rho) (EMBED_FS_PLOY_Func with
// A = -1, zero for rho <= 0).  The reader sets neither RMAX nor RHOMX, so the grid runs to the
// cutoff and RHOD = RHOSCAL * max POTB / NEMBD (Create_Pairwise_ForceTable).
namespace {

bool moldy_numbers(FILE *f, std::vector<double> &v)
{
    char buf[8192];
    if (!fgets(buf, sizeof(buf), f)) return false;
    v.clear();
    std::string tok;
    for (const char *p = buf;; ++p) {
        const char c = *p;
        const bool sep = c == '\0' || c == ' ' || c == '\t' || c == ',' || c == '(' || c == ')' || c == '[' ||
                         c == ']' || c == '{' || c == '}' || c == '=' || c == '\n' || c == '\r';
        if (sep) {
            if (!tok.empty()) {
                char *end = nullptr;
                const double x = strtod(tok.c_str(), &end);
                if (end != tok.c_str() && *end == '\0') v.push_back(x);
                tok.clear();
            }
            if (c == '\0') break;
        } else {
            tok.push_back(c);
        }
    }
    return true;
}

}  // namespace

extern "C" int msmgb_moldy_tables(const char *path, double rmax, int ntab, int nembd, double rhoscal,
                                  double *potr, double *fpotr, double *potb, double *fpotb, double *fembd,
                                  double *dfembd, double *rhod)
{
    if (!path || rmax <= 0.0 || ntab < 2 || nembd < 2 || !potr || !fpotr || !potb || !fpotb || !fembd ||
        !dfembd)
        return MSMGB_ERR_ARG;
    if (!(rhoscal > 0.0)) rhoscal = 20.0;
    FILE *f = fopen(path, "r");
    if (!f) return MSMGB_ERR_ARG;
    char sym[256];
    std::vector<double> av, rv, ab, rb, cst;
    const bool ok = fgets(sym, sizeof(sym), f) && moldy_numbers(f, av) && moldy_numbers(f, rv) &&
                    moldy_numbers(f, ab) && moldy_numbers(f, rb) && moldy_numbers(f, cst);
    fclose(f);
    if (!ok || av.empty() || av.size() != rv.size() || ab.empty() || ab.size() != rb.size() || cst.empty() ||
        !(cst[0] > 0.0))
        return MSMGB_ERR_ARG;
    const double a0 = cst[0];
    for (double &x : rv) x *= a0;
    for (double &x : rb) x *= a0;
    for (double &x : av) x /= std::pow(a0, 3.0);
    for (double &x : ab) x /= std::pow(a0, 6.0);
    const double csiv = std::sqrt(rmax) / ntab;
    double rhomx = 0.0;
    for (int i = 1; i <= ntab; ++i) {
        const double t = i * csiv, r = t * t;
        double v, dv, b, db;
        cubic_knots(r, av.data(), rv.data(), (int)av.size(), &v, &dv);
        cubic_knots(r, ab.data(), rb.data(), (int)ab.size(), &b, &db);
        potr[i - 1] = 0.5 * v * r;
        fpotr[i - 1] = dv * r;
        potb[i - 1] = b;
        fpotb[i - 1] = db;
        if (rhomx < b * rhoscal) rhomx = b * rhoscal;
    }
    const double d = rhomx / nembd;
    for (int i = 1; i <= nembd; ++i) {
        const double rho = (i - 1) * d;
        fembd[i - 1] = rho > 0.0 ? -std::sqrt(rho) : 0.0;
        dfembd[i - 1] = rho > 0.0 ? -0.5 / std::sqrt(rho) : 0.0;
    }
    if (rhod) *rhod = d;
    return MSMGB_OK;
}

// ---- tables exported by the reference and read back (Export_ForceTable, Import_ForceTable,
//      Register_Imported_ForceTable; MD_TypeDef_ForceTable.F90:1315-1459, 1463-1608, 1612-1855)
//
// The reference runs every potential it cannot generate itself (the NIST files, and any
// library name with no built-in generator) from a pair of text files `stem.pair` and
// `stem.embd` (MD_ForceLib_Register.F90:405-420): a header with &POTTYPE, &NUMTABLE (the
// table ids) and &NUMPOINT, then one row per grid point.  Pair rows: index, r [A], and per
// table 2 r V [eV A], -r dV/dr [eV], rho (FS: eV^2), -drho/dr [/A]; embedding rows: index,
// rho, and per table F [eV], dF/drho (CGS: erg per rho unit; FS: 1/(2 F) in 1/erg).  The
// import re-grids every column the box needs onto the run's sqrt(r) grid (T = K CSIV, CSIV =
// 1/CSI, CSI = NTAB/sqrt(Rmax); value 0 where T^2 exceeds the file's largest r) and the
// embedding columns onto rho = (K-1) RHOD with RHOMX = RHO(N) N/(N-1), RHOD = RHOMX/NEMBD,
// through SPLID1/SPLID2 (LIB/sor/f/MiniUtilities/DINTF2.F:17-240) with IOP = 5 at both ends:
// the cubic spline through the rows whose end slopes are those of the cubic through the
// first (last) four rows, extended beyond the end rows by the end intervals' cubics.  Here
// that spline is computed in slope (Hermite) form: one tridiagonal solve for the knot slopes.
namespace {

const double kA2CM = 1e-8;   // MSM_Const.F90:67

struct ImpFile {
    std::string pottype;
    std::vector<int> ids;                    // table ids (FPAIR / FPAIR1) in file order
    int npt = 0;
    std::vector<double> x;                   // r or rho per row
    std::vector<std::vector<double>> col;    // [table * ncol + c][row]
};

std::string upcase(std::string s)
{
    for (char &ch : s) ch = (char)toupper((unsigned char)ch);
    return s;
}

// header keywords of Import_ForceTable (:1485-1512) and the rows after "&#"
int read_imported(const char *path, int ncol, ImpFile &f, std::string &why)
{
    FILE *fh = fopen(path, "r");
    if (!fh) {
        why = std::string("cannot open ") + path;
        return MSMGB_ERR_ARG;
    }
    char buf[65536];
    bool header_done = false;
    int nc = -1;
    while (fgets(buf, sizeof(buf), fh)) {
        std::string s = trim(buf);
        if (s.empty() || s[0] == '!') continue;
        if (s[0] != '&') continue;
        const size_t sp = s.find_first_of(" \t");
        const std::string key = upcase(s.substr(0, sp));
        const std::string rest = sp == std::string::npos ? std::string() : s.substr(sp);
        if (key == "&NUMTABLE") {
            std::vector<int> nums;
            const char *p = rest.c_str();
            while (*p) {
                if (isdigit((unsigned char)*p)) {
                    char *e = nullptr;
                    nums.push_back((int)strtol(p, &e, 10));
                    p = e;
                } else {
                    ++p;
                }
            }
            if (nums.empty() || nums[0] < 1 || (int)nums.size() < nums[0] + 1) break;
            nc = nums[0];
            f.ids.assign(nums.begin() + 1, nums.begin() + 1 + nc);
        } else if (key == "&NUMPOINT") {
            f.npt = atoi(rest.c_str());
        } else if (key == "&POTTYPE") {
            const std::vector<std::string> q = quoted(rest);
            f.pottype = q.empty() ? trim(rest) : q[0];
        } else if (key.compare(0, 2, "&#") == 0) {
            header_done = true;
            break;
        }
    }
    if (!header_done || nc < 1 || f.npt < 4) {
        fclose(fh);
        why = std::string("bad header (need &NUMTABLE, &NUMPOINT >= 4 and the &# line) in ") + path;
        return MSMGB_ERR_ARG;
    }
    f.x.assign((size_t)f.npt, 0.0);
    f.col.assign((size_t)nc * ncol, std::vector<double>((size_t)f.npt, 0.0));
    std::string t;
    for (int r = 0; r < f.npt; ++r) {
        for (int c = -1; c < nc * ncol + 1; ++c) {          // index, x, then the table columns
            char *e = nullptr;
            if (!next_token(fh, t)) goto short_file;
            const double v = strtod(t.c_str(), &e);
            if (e == t.c_str()) goto short_file;
            if (c == 0) f.x[(size_t)r] = v;
            else if (c > 0) f.col[(size_t)(c - 1)][(size_t)r] = v;
        }
    }
    fclose(fh);
    for (int r = 1; r < f.npt; ++r)
        if (!(f.x[(size_t)r] > f.x[(size_t)r - 1])) {
            why = std::string("grid not increasing in ") + path;
            return MSMGB_ERR_ARG;
        }
    return MSMGB_OK;
short_file:
    fclose(fh);
    why = std::string("fewer rows than &NUMPOINT in ") + path;
    return MSMGB_ERR_ARG;
}

// slope of the cubic through (x[i0..i0+3], y[..]) at x[at] (Lagrange form)
double lagrange4_slope(const double *x, const double *y, int at)
{
    double s = 0.0;
    for (int j = 0; j < 4; ++j) {
        if (j == at) {
            double w = 0.0;
            for (int k = 0; k < 4; ++k)
                if (k != at) w += 1.0 / (x[at] - x[k]);
            s += y[j] * w;
        } else {
            double num = 1.0, den = 1.0;
            for (int k = 0; k < 4; ++k) {
                if (k != j) den *= x[j] - x[k];
                if (k != j && k != at) num *= x[at] - x[k];
            }
            s += y[j] * num / den;
        }
    }
    return s;
}

// Clamped cubic spline in Hermite form: knot slopes d_i with d_0, d_{n-1} given and, inside,
// h_i d_{i-1} + 2 (h_{i-1} + h_i) d_i + h_{i-1} d_{i+1} = 3 (h_i D_{i-1} + h_{i-1} D_i),
// D_i = (y_{i+1} - y_i) / h_i, h_i = x_{i+1} - x_i (continuity of the second derivative).
struct HSpline {
    const double *x = nullptr, *y = nullptr;
    int n = 0;
    std::vector<double> d;
};

void hspline_build(HSpline &s, const double *x, const double *y, int n)
{
    s.x = x;
    s.y = y;
    s.n = n;
    s.d.assign((size_t)n, 0.0);
    s.d[0] = lagrange4_slope(x, y, 0);
    s.d[(size_t)n - 1] = lagrange4_slope(x + n - 4, y + n - 4, 3);
    std::vector<double> cp((size_t)n, 0.0), rp((size_t)n, 0.0);
    // forward elimination of the interior rows (unknowns d_1..d_{n-2})
    for (int i = 1; i <= n - 2; ++i) {
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        const double D0 = (y[i] - y[i - 1]) / h0, D1 = (y[i + 1] - y[i]) / h1;
        const double a = h1, b = 2.0 * (h0 + h1), c = h0;
        double r = 3.0 * (h1 * D0 + h0 * D1);
        if (i == 1) r -= a * s.d[0];
        if (i == n - 2) r -= c * s.d[(size_t)n - 1];
        const double den = b - (i > 1 ? a * cp[(size_t)i - 1] : 0.0);
        cp[(size_t)i] = (i < n - 2) ? c / den : 0.0;
        rp[(size_t)i] = (r - (i > 1 ? a * rp[(size_t)i - 1] : 0.0)) / den;
    }
    for (int i = n - 2; i >= 1; --i)
        s.d[(size_t)i] = rp[(size_t)i] - (i < n - 2 ? cp[(size_t)i] * s.d[(size_t)i + 1] : 0.0);
}

// value at t: the interval x_i <= t < x_{i+1}; below x_0 the first, from x_{n-1} on the last
// interval's cubic (SPLID2's interval choice)
double hspline_at(const HSpline &s, double t)
{
    int lo = 0, hi = s.n - 1;
    if (t <= s.x[0]) {
        hi = 1;
    } else if (t >= s.x[s.n - 1]) {
        lo = s.n - 2;
    } else {
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (s.x[mid] <= t) lo = mid; else hi = mid;
        }
    }
    const double h = s.x[hi] - s.x[lo], u = (t - s.x[lo]) / h;
    const double u2 = u * u, u3 = u2 * u;
    const double h00 = 2.0 * u3 - 3.0 * u2 + 1.0, h10 = u3 - 2.0 * u2 + u;
    const double h01 = -2.0 * u3 + 3.0 * u2, h11 = u3 - u2;
    return h00 * s.y[lo] + h10 * h * s.d[(size_t)lo] + h01 * s.y[hi] + h11 * h * s.d[(size_t)hi];
}

// first-appearance numbering of PTYPE(I,J) (I outer, J inner; New_ForceTable :560-574)
void number_tables(int ng, const int *ptype, bool diag, std::vector<int> &ids, std::vector<int> &k)
{
    ids.clear();
    k.assign((size_t)ng * ng, 0);
    for (int i = 0; i < ng; ++i)
        for (int j = 0; j < ng; ++j) {
            if (diag && i != j) continue;
            const int id = ptype[(size_t)j * ng + i];          // PTYPE(I,J), column-major
            size_t q = 0;
            while (q < ids.size() && ids[q] != id) ++q;
            if (q == ids.size()) ids.push_back(id);
            k[(size_t)j * ng + i] = (int)q + 1;
        }
}

int file_table(const ImpFile &f, int id)
{
    for (size_t q = 0; q < f.ids.size(); ++q)
        if (f.ids[q] == id) return (int)q;
    return -1;
}

}  // namespace

extern "C" int msmgb_import_info(const char *stem, int *pottype, int *ntables, int *ids, int *npoint,
                                 int *nembtables, int *emb_ids, int *nembpoint)
{
    if (!stem) return MSMGB_ERR_ARG;
    ImpFile p, e;
    std::string why;
    if (read_imported((std::string(stem) + ".pair").c_str(), 4, p, why) != MSMGB_OK) return MSMGB_ERR_ARG;
    if (read_imported((std::string(stem) + ".embd").c_str(), 2, e, why) != MSMGB_OK) return MSMGB_ERR_ARG;
    const std::string pt = upcase(p.pottype);
    if (pottype) *pottype = pt == "EAM_TYPE" ? MSMGB_EAM_TYPE : MSMGB_FS_TYPE;
    if (ntables) *ntables = (int)p.ids.size();
    if (ids) for (size_t q = 0; q < p.ids.size(); ++q) ids[q] = p.ids[q];
    if (npoint) *npoint = p.npt;
    if (nembtables) *nembtables = (int)e.ids.size();
    if (emb_ids) for (size_t q = 0; q < e.ids.size(); ++q) emb_ids[q] = e.ids[q];
    if (nembpoint) *nembpoint = e.npt;
    return MSMGB_OK;
}

extern "C" int msmgb_import_forcetable(const char *stem, int units, int ngroup, const int *ptype, double rmax,
                                       int ntab, int nembd, double *potr, double *fpotr, double *potb,
                                       double *fpotb, double *fembd, double *dfembd, int *kpair, int *kembd,
                                       int *nkind, int *nkind1, double *rhod, int *pottype)
{
    if (!stem || !ptype || ngroup < 1 || ngroup > 16 || !(rmax > 0.0) || ntab < 2 || !potr || !fpotr || !potb ||
        !fpotb || !kpair || (units != MSMGB_UNITS_EV_A && units != MSMGB_UNITS_CGS))
        return MSMGB_ERR_ARG;
    ImpFile p, e;
    std::string why;
    if (read_imported((std::string(stem) + ".pair").c_str(), 4, p, why) != MSMGB_OK) return MSMGB_ERR_ARG;
    if (read_imported((std::string(stem) + ".embd").c_str(), 2, e, why) != MSMGB_OK) return MSMGB_ERR_ARG;
    const bool eam = upcase(p.pottype) == "EAM_TYPE";
    if (eam && (nembd < 2 || !fembd || !dfembd || !kembd)) return MSMGB_ERR_ARG;
    // every table the box names must be in both files (:1631-1651)
    for (int q = 0; q < ngroup * ngroup; ++q)
        if (file_table(p, ptype[q]) < 0) return MSMGB_ERR_ARG;
    for (int i = 0; i < ngroup; ++i)
        if (file_table(e, ptype[(size_t)i * ngroup + i]) < 0) return MSMGB_ERR_ARG;
    // unit conversion of Import_ForceTable (:1529-1540, 1583-1585); the files are in A / eV
    const bool cgs = units == MSMGB_UNITS_CGS;
    const double rhounit = (!eam && cgs) ? 1.0 / (kEVERG * kEVERG) : 1.0;
    const double fx = cgs ? kA2CM : 1.0;
    const double fc[4] = {0.5 * (cgs ? kEVERG * kA2CM : 1.0), cgs ? kEVERG : 1.0, 1.0 / rhounit,
                          (cgs ? 1.0 / kA2CM : 1.0) / rhounit};
    for (double &v : p.x) v *= fx;
    for (size_t q = 0; q < p.ids.size(); ++q)
        for (int c = 0; c < 4; ++c)
            for (double &v : p.col[q * 4 + c]) v *= fc[c];
    for (double &v : e.x) v /= rhounit;
    for (size_t q = 0; q < e.ids.size(); ++q) {
        for (double &v : e.col[q * 2]) v *= cgs ? kEVERG : 1.0;
        if (!cgs)
            for (double &v : e.col[q * 2 + 1]) v /= kEVERG;   // the file keeps dF/drho in CGS
    }
    // pair tables the box needs, first-appearance order, re-gridded (:1667-1760)
    std::vector<int> ids, kp;
    number_tables(ngroup, ptype, false, ids, kp);
    const int nk = (int)ids.size();
    const double csi = (double)ntab / std::sqrt(rmax), csiv = 1.0 / csi;
    double trmax = p.x[0];
    for (double v : p.x) trmax = std::max(trmax, v);
    double *dst[4] = {potr, fpotr, potb, fpotb};
    for (int k = 0; k < nk; ++k) {
        const int q = file_table(p, ids[(size_t)k]);
        for (int c = 0; c < 4; ++c) {
            HSpline s;
            hspline_build(s, p.x.data(), p.col[(size_t)q * 4 + c].data(), p.npt);
            for (int i = 1; i <= ntab; ++i) {
                const double t = (double)i * csiv, tt = t * t;
                dst[c][(size_t)(i - 1) * nk + k] = tt <= trmax ? hspline_at(s, tt) : 0.0;
            }
        }
    }
    for (int q = 0; q < ngroup * ngroup; ++q) kpair[q] = kp[(size_t)q];
    if (nkind) *nkind = nk;
    if (pottype) *pottype = eam ? MSMGB_EAM_TYPE : MSMGB_FS_TYPE;
    // embedding tables of the groups (:1785-1838); FS potentials have none
    const int ne = e.npt;
    double rmx = (e.x[(size_t)ne - 1] / (double)(ne - 1)) * (double)ne;
    double rd = nembd > 0 ? rmx / (double)nembd : 1.0;
    if (rd <= 1e-64) rd = 1.0;
    if (rhod) *rhod = rd;
    if (!eam) {
        if (nkind1) *nkind1 = 0;
        return MSMGB_OK;
    }
    std::vector<int> eids, ke;
    number_tables(ngroup, ptype, true, eids, ke);
    const int nk1 = (int)eids.size();
    for (int k = 0; k < nk1; ++k) {
        const int q = file_table(e, eids[(size_t)k]);
        double *edst[2] = {fembd, dfembd};
        for (int c = 0; c < 2; ++c) {
            HSpline s;
            hspline_build(s, e.x.data(), e.col[(size_t)q * 2 + c].data(), ne);
            for (int i = 1; i <= nembd; ++i)
                edst[c][(size_t)(i - 1) * nk1 + k] = hspline_at(s, (double)(i - 1) * rd);
        }
    }
    for (int i = 0; i < ngroup; ++i) kembd[i] = ke[(size_t)i * ngroup + i];
    if (nkind1) *nkind1 = nk1;
    return MSMGB_OK;
}

// Export_ForceTable (:1315-1459): the two files in the reference's layout and number format
// (1PE21.9 pair columns, 1PE16.8 embedding columns), tables in increasing id order.
extern "C" int msmgb_export_forcetable(const char *stem, int units, const msmgb_forcetable *ft, const int *ids,
                                       const int *emb_ids)
{
    if (!stem || !ft || !ft->potr || !ft->fpotr || !ft->potb || !ft->fpotb || ft->ntab < 1 || ft->nkind < 1 ||
        !(ft->rmax > 0.0) || (units != MSMGB_UNITS_EV_A && units != MSMGB_UNITS_CGS))
        return MSMGB_ERR_ARG;
    const bool eam = ft->pottype == MSMGB_EAM_TYPE;
    if (eam && (ft->nembd < 1 || ft->nkind1 < 1 || !ft->fembd || !ft->dfembd)) return MSMGB_ERR_ARG;
    const bool cgs = units == MSMGB_UNITS_CGS;
    const double rhounit = (!eam && cgs) ? 1.0 / (kEVERG * kEVERG) : 1.0;
    const int nk = ft->nkind;
    std::vector<int> id((size_t)nk), tid((size_t)nk);
    for (int k = 0; k < nk; ++k) id[(size_t)k] = ids ? ids[k] : k + 1;
    for (int k = 0; k < nk; ++k) tid[(size_t)k] = k;
    std::stable_sort(tid.begin(), tid.end(), [&](int a, int b) { return id[(size_t)a] < id[(size_t)b]; });
    const char *ptn = eam ? "EAM_TYPE" : "FS_TYPE";
    FILE *f = fopen((std::string(stem) + ".pair").c_str(), "w");
    if (!f) return MSMGB_ERR_ARG;
    fprintf(f, "&MDPSCU_POTTAB.Pair\n !     exported by libmsmgb (msmgb_export_forcetable)\n");
    fprintf(f, "!     \n!     NOTE: For FS potential, RHO is in eV^2, the potential calculated by\n"
               "!           -sqrt(RHO)+V(r) \n!           is thus in unit eV, and the d(RHO)/dr in unit eV^2/A.\n"
               "!           \n!           For EAM potential, not specific unit is assigned for RHO,\n"
               "!           and for d(RHO)/dr. The potential calculated by \n"
               "!           F(RHO)+V(r) is in unit eV.\n!           \n");
    fprintf(f, "&POTTYPE \"%s\"\n&NUMTABLE %7d table IDs: ", ptn, nk);
    for (int k = 0; k < nk; ++k) fprintf(f, "%5d", id[(size_t)tid[(size_t)k]]);
    fprintf(f, "\n&NUMPOINT %7d\n&#     ", ft->ntab);
    fprintf(f, "      Rij(A)     ");
    for (int k = 0; k < nk; ++k) {
        const int j = id[(size_t)tid[(size_t)k]];
        fprintf(f, "      r*V%d(r)[eV*A]        -r*dV%d/dr[eV]            RHO%d(r)            -dRHO%d/dr[/A] ", j, j,
                j, j);
    }
    fprintf(f, "\n");
    const double csi = (double)ft->ntab / std::sqrt(ft->rmax), csiv = 1.0 / csi;
    for (int i = 1; i <= ft->ntab; ++i) {
        const double t = (double)i * csiv;
        fprintf(f, " %6d %21.9E", i, (t * t) * (cgs ? 1.0 / kA2CM : 1.0));
        for (int k = 0; k < nk; ++k) {
            const size_t o = (size_t)(i - 1) * nk + tid[(size_t)k];
            fprintf(f, "%21.9E%21.9E%21.9E%21.9E", ft->potr[o] * 2.0 * (cgs ? 1.0 / (kEVERG * kA2CM) : 1.0),
                    ft->fpotr[o] * (cgs ? 1.0 / kEVERG : 1.0), ft->potb[o] * rhounit,
                    ft->fpotb[o] * rhounit * (cgs ? kA2CM : 1.0));
        }
        fprintf(f, "\n");
    }
    if (fclose(f) != 0) return MSMGB_ERR_ARG;
    // embedding file
    const int nk1 = eam ? ft->nkind1 : 1;
    std::vector<int> eid((size_t)nk1), etid((size_t)nk1);
    for (int k = 0; k < nk1; ++k) eid[(size_t)k] = (eam && emb_ids) ? emb_ids[k] : k + 1;
    for (int k = 0; k < nk1; ++k) etid[(size_t)k] = k;
    std::stable_sort(etid.begin(), etid.end(), [&](int a, int b) { return eid[(size_t)a] < eid[(size_t)b]; });
    f = fopen((std::string(stem) + ".embd").c_str(), "w");
    if (!f) return MSMGB_ERR_ARG;
    fprintf(f, "&MDPSCU_POTTAB.Embd\n !     exported by libmsmgb (msmgb_export_forcetable)\n");
    fprintf(f, "&POTTYPE \"%s\"\n&NUMTABLE %7d table IDs: ", ptn, nk1);
    for (int k = 0; k < nk1; ++k) fprintf(f, "%5d", eid[(size_t)etid[(size_t)k]]);
    const int ne = eam ? ft->nembd : ft->ntab;
    fprintf(f, "\n&NUMPOINT %7d\n&#     ", ne);
    fprintf(f, "      RHO      ");
    for (int k = 0; k < nk1; ++k) {
        const int j = eid[(size_t)etid[(size_t)k]];
        fprintf(f, "         F%d(RHO)      dF%d/d(RHO)", j, j);
    }
    fprintf(f, "\n");
    // FS: RHOD of the density tables (Create_EMBDFUNTable); the column is informational
    double rd = ft->rhod;
    for (int i = 1; i <= ne; ++i) {
        const double r = (double)(i - 1) * rd * rhounit;    // file rho (FS: eV^2)
        fprintf(f, " %6d %16.8E", i, r);
        for (int k = 0; k < nk1; ++k) {
            double den, deni;
            if (!eam) {
                // DEN = -sqrt(rho)/ERGEV in erg, DENI = 1/(2 DEN) (:1444-1449)
                den = r > 0.0 ? -std::sqrt(r) * kEVERG : 0.0;
                deni = r > 0.0 ? 0.5 / den : 0.0;
            } else {
                const size_t o = (size_t)(i - 1) * nk1 + etid[(size_t)k];
                den = ft->fembd[o] * (cgs ? 1.0 : kEVERG);      // erg
                deni = ft->dfembd[o] * (cgs ? 1.0 : kEVERG);    // CGS per rho unit
            }
            fprintf(f, "%16.8E%16.8E", den / kEVERG, deni);
        }
        fprintf(f, "\n");
    }
    if (fclose(f) != 0) return MSMGB_ERR_ARG;
    return MSMGB_OK;
}
