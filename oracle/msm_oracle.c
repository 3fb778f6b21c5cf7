/*
 * msm_oracle.c -- CPU restatement of msmpscu's many-body (FS / EAM) force path, its cell
 * neighbour list and its Swope velocity-Verlet integrator.
 *
 * TEST INFRASTRUCTURE ONLY.  It is the checker for the CUDA library and the CPU baseline
 * that bench.py times; nothing in the product links or calls it.
 *
 * Parity status: the table generator is pinned by the reference's exported table fixture
 * (see tests/golden/); the force and per-atom energy evaluation reproduces the reference's
 * own output for a 2,001-atom W + H box (its NEB example's step-0 GMD records,
 * tests/golden/make_golden_neb.py) to the records' printed digits; lists, virial and
 * trajectories have no reference record and are a statement-level restatement ("parity
 * unpinned" there).
 *
 * Deliberate deviations from the reference, each cited where it happens:
 *   - the cell list uses minimum-image distances, so boxes whose cells are smaller than
 *       the list cutoff (NCELL forced to 3) still find every neighbour;
 *   - the tables are read as if padded: index NTAB+1 returns T(NTAB) (only ever hit with
 *       DK = 0), index 0 returns 0;
 *   - the full-list force pairs FPOTB(KPAIR(I,J)) with DEN(I), as the GPU kernels do.
 * Compile with -ffp-contract=off so x86 and Arm give identical results.
 */
#include "msm_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------ */
/* potential functions (Angstrom / eV)                                                   */
/* ------------------------------------------------------------------------------------ */

/* Cleri-Rosato pair and density terms, TB_CR_AuAu.F90:22-35 and 38-56:
 *   POTR  = A exp(-p (r/r0 - 1)),      FPOTR = 2 POTR p/r0   (= 2 (-V'))
 *   POTB  = xi^2 exp(-2q (r/r0 - 1)),  FPOTB = POTB q/r0 * 2 (= -rho')            */
static void cr_nn(double r, const double *prm, double *potr, double *fpotr)
{
    const double A = prm[0], P = prm[2], r0 = prm[4];
    const double psr0 = P / r0;
    double v = A * exp(-P * ((r / r0) - 1.0));
    *potr = v;
    *fpotr = 2.0 * v * psr0;
}

static void cr_ne(double r, const double *prm, double *potb, double *fpotb)
{
    const double xi = prm[1], Q = prm[3], r0 = prm[4];
    const double qsr0 = Q / r0, eta2 = xi * xi, twoq = 2.0 * Q;
    double rho = eta2 * exp(-twoq * ((r / r0) - 1.0));
    *potb = rho;
    *fpotb = rho * qsr0 * 2.0;
}

/* Marinica EAM2/EAM3/EAM4 W (EAM2_WW_Marinica_JPCM25_2013.F90:17-116 and the EAM3, EAM4
 * files of the same folder) through the cubic-knot helpers of MD_Pot_EAM_Utilities.F90:48-85
 * (returns 0.5 V and -V') and 259-290 (rho, -rho').  Literals written without a D exponent
 * in the reference are default REAL, i.e. single precision; those are given here as float
 * literals (f suffix) and widened: EAM2's knot radii, EAM3's knot radii and embedding
 * coefficients, EAM4's pair knot radii. */
typedef struct {
    int nv;
    double a[15], r[15];      /* pair knots */
    double b[4], rb[4];       /* density knots */
    double f[2];              /* embedding: f1 sqrt(rho) + f2 rho^2 */
} mar_set_t;

static const double mar_rc = 2.002970124727;

static const mar_set_t mar_sets[3] = {
    {15,
     {0.960851701343041e2, -0.184410923895214e3, 0.935784079613550e2, -0.798358265041677e1,
      0.747034092936229e1, -0.152756043708453e1, 0.125205932634393e1, 0.163082162159425e1,
      -0.141854775352260e1, -0.819936046256149e0, 0.198013514305908e1, -0.696430179520267e0,
      0.304546909722160e-1, -0.163131143161660e1, 0.138409896486177e1},
     {2.564897500000000f, 2.629795000000000f, 2.694692500000000f, 2.866317500000000f,
      2.973045000000000f, 3.079772500000000f, 3.516472500000000f, 3.846445000000000f,
      4.176417500000000f, 4.700845000000000f, 4.895300000000000f, 5.089755000000000f,
      5.342952500000000f, 5.401695000000000f, 5.460437500000000f},
     {-0.420429107805055e1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.500000000000000f, 3.100000000000000f, 3.500000000000000f, 4.900000000000000f},
     {-5.946454472402710, -0.049477376935239}},
    {14,
     {0.335180090207171e3, -0.630187843239795e3, 0.351436490059390e3, -0.187104554936536e-1,
      0.599698179163370e-1, -0.210635074070024e-1, 0.258575483268791e-1, 0.389896994857220e-1,
      -0.139737073858817e-1, 0.184785876328131e-1, -0.505971175928021e0, -0.890738292956047e1,
      0.495992901621487e-1, 0.377639491131043e-1},
     {2.610000000000000f, 2.680000000000000f, 2.718160253915930f, 2.758522910939240f,
      2.892427681390960f, 3.401517108884100f, 3.675283167162630f, 4.248392613157640f,
      4.631029170086540f, 4.822645095086770f, 5.021214835934140f, 5.282885848627100f,
      5.283029247305360f, 5.290925630219230f},
     {-0.420429107805055e-1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.500000000000000f, 3.100000000000000f, 3.500000000000000f, 4.900000000000000f},
     {-5.073237905708500f, -0.039263610952181f}},
    {15,
     {0.954071477542914e2, -0.181161004448916e3, 0.930215233132627e2, -0.108428907515182e2,
      0.112027468539573e2, -0.312459176640227e1, 0.123028140617302e1, 0.154767467307454e1,
      -0.128861387780439e1, -0.843327493551467e0, 0.214009882965042e1, -0.102898314532388e1,
      0.138163259601912e1, -0.360872433001551e1, 0.217655968740690e1},
     {2.564897500000000f, 2.629795000000000f, 2.694692500000000f, 2.866317500000000f,
      2.973045000000000f, 3.079772500000000f, 3.516472500000000f, 3.846445000000000f,
      4.176417500000000f, 4.700845000000000f, 4.895300000000000f, 5.089755000000000f,
      5.342952500000000f, 5.401695000000000f, 5.460437500000000f},
     {-0.420429107805055e-1, 0.518217702261442e0, 0.562720834534370e-1, 0.344164178842340e-1},
     {2.5, 3.1, 3.5, 4.9},
     {-5.553986589859130, -0.045691157657292}}};

static double step_h(double x) { return x >= 0.0 ? 1.0 : 0.0; }   /* MD_Pot_EAM_Utilities.F90:35-44 */

static void mar_set_nn(const mar_set_t *m, double rt, double *potr, double *fpotr)
{
    double p = 0.0, f = 0.0;
    for (int i = 0; i < m->nv; ++i) {
        const double ri = m->r[i], stp = step_h(ri - rt);
        p = p + m->a[i] * (ri - rt) * (ri - rt) * (ri - rt) * stp;
        f = f + m->a[i] * (ri - rt) * (ri - rt) * stp;
    }
    *potr = 0.5 * p;
    *fpotr = 3.0 * f;
}

static void mar_set_rho(const mar_set_t *m, double rt, double *potb, double *fpotb)
{
    double p = 0.0, f = 0.0;
    for (int i = 0; i < 4; ++i) {
        const double ri = m->rb[i], stp = step_h(ri - rt);
        p = p + m->b[i] * (ri - rt) * (ri - rt) * (ri - rt) * stp;
        f = f + m->b[i] * (ri - rt) * (ri - rt) * stp;
    }
    *potb = p;
    *fpotb = 3.0 * f;
}

/* density frozen inside RC (EAM2_WW_Marinica_JPCM25_2013.F90:83-88, the same in EAM3/EAM4) */
static void mar_set_ne(const mar_set_t *m, double r, double *potb, double *fpotb)
{
    if (r <= mar_rc) {
        mar_set_rho(m, mar_rc, potb, fpotb);
        *fpotb = 0.0;
    } else {
        mar_set_rho(m, r, potb, fpotb);
    }
}

/* EMBED_FS_PLOY_Func, MD_Pot_EAM_Utilities.F90:332-368: F = a1 sqrt(rho) + a2 rho^2 */
static void mar_set_embed(const mar_set_t *m, double rho, double *f, double *df)
{
    if (rho <= 0.0) { *f = 0.0; *df = 0.0; return; }
    double trho = rho;
    double fr = m->f[0] * sqrt(trho);
    double dfr = 0.5 * m->f[0] / sqrt(trho);
    fr = fr + m->f[1] * rho * trho;
    dfr = dfr + 2.0 * m->f[1] * trho;
    *f = fr;
    *df = dfr;
}

static void mar_nn(double r, double *potr, double *fpotr) { mar_set_nn(&mar_sets[0], r, potr, fpotr); }
static void mar_ne(double r, double *potb, double *fpotb) { mar_set_ne(&mar_sets[0], r, potb, fpotb); }
static void mar_embed(double rho, double *f, double *df) { mar_set_embed(&mar_sets[0], rho, f, df); }

/* Ackland-Thetford W-W (FS form), EM_TB_WangJun_W-HE_2010/FS_Ackland_WW.F90:23-88, restated
 * in Angstrom / eV (the reference's CGS constants divided out). */
static void ack_nn(double r, double *potr, double *fpotr)
{
    const double c = 3.25, c0 = 47.1346499, c1 = -33.7665655, c2 = 6.2541999;
    const double ackb = 90.3, acka = 1.2, ackb0 = 2.7411;
    double fs = 0.0, dfs = 0.0;
    if (r < ackb0) {
        fs = ackb * pow(ackb0 - r, 3.0) * exp(-acka * r);
        dfs = -ackb * (3.0 * pow(ackb0 - r, 2.0) * exp(-acka * r) +
                       acka * pow(ackb0 - r, 3.0) * exp(-acka * r));
    }
    if (r <= c) {
        double p = pow(r - c, 2.0) * (c0 + c1 * r + c2 * pow(r, 2.0)) + fs;
        double f = 2.0 * (r - c) * (c0 + c1 * r + c2 * pow(r, 2.0)) +
                   pow(r - c, 2.0) * (c1 + 2.0 * c2 * r) + dfs;
        *potr = 0.5 * p;
        *fpotr = -f;
    } else {
        *potr = 0.0;
        *fpotr = 0.0;
    }
}

static void ack_ne(double r, double *potb, double *fpotb)
{
    const double a = 1.896373, d = 4.400224;
    if (r <= d) {
        *potb = a * a * pow(r - d, 2.0);
        *fpotb = -(a * a * 2.0 * (r - d));
    } else {
        *potb = 0.0;
        *fpotb = 0.0;
    }
}

/* Derlet-Nguyen-Manh-Dudarev W (FS form), EM_TB_WangJun_W-HE_2010/FS_PM_WW.F90:7-204, restated
 * in Angstrom / eV: knots x1e8, pair coefficients (erg/cm^3 / CP_EVERG) x1e-24 eV/A^3, density
 * coefficients x1e-24 /A^3.  The prefactor A (:13) has no exponent letter in the source, so the
 * reference holds it as a single-precision number: (float)10.84238200368439 eV. */
static void der_nn(double r, double *potr, double *fpotr)
{
    static const double kn[9] = {4.2689, 3.98568, 3.70246, 3.41924, 3.13602, 2.8528, 2.74110,
                                 2.604045, 2.46699};
    static const double cv[9] = {-0.1036435865158945, -0.2912948318493851, -2.096765499656263,
                                 19.1604545270101, -41.01619862085917, 46.05205617244703,
                                 26.42203930654883, 15.35211507804088, 14.12806259323987};
    double v = 0.0, dv = 0.0;
    for (int k = 0; k < 9; ++k) {
        if (r > kn[k]) continue;
        v += cv[k] * pow(kn[k] - r, 3.0);
        dv += 3.0 * cv[k] * pow(kn[k] - r, 2.0);
    }
    *potr = 0.5 * v;
    *fpotr = dv;
}

static void der_ne(double r, double *potb, double *fpotb)
{
    static const double kn[7] = {3.3216, 3.165333333333333, 3.009066666666667, 2.8528, 2.7411,
                                 2.604045, 2.46699};
    static const double cf[7] = {1.677334871575606, -1.673137509507131, -4.737051994974169,
                                 7.870789420780674, -3.7924230525563378e-4, 6.190816158916646,
                                 -0.9565713891199151};
    const double a = (double)(float)10.84238200368439;
    double p = 0.0, d = 0.0;
    for (int k = 0; k < 7; ++k) {
        if (r > kn[k]) continue;
        p += cf[k] * pow(kn[k] - r, 3.0);
        d += 3.0 * cf[k] * pow(kn[k] - r, 2.0);
    }
    *potb = a * a * p;
    *fpotb = a * a * d;
}

/* ZBL universal screening phi(x) and -dphi/dx */
static void zbl_phi(double x, double *phi, double *mdphi)
{
    static const double c[4] = {0.18175, 0.50986, 0.28022, 0.028171};
    static const double b[4] = {3.1998, 0.94229, 0.4029, 0.20162};
    *phi = 0.0;
    *mdphi = 0.0;
    for (int k = 0; k < 4; ++k) {
        *phi += c[k] * exp(-b[k] * x);
        *mdphi += b[k] * c[k] * exp(-b[k] * x);
    }
}

/* He-He, ZBL_EXP6_HeHe.F90:7-86 (ZBL of MD_CorePotent.F90:24-75 below 1 A, its fitted cubic to
 * 1.3 A, EXP6 beyond), in Angstrom / eV.  The ZBL Coulomb constant 9e9 qe^2 (SI, :37-39) is
 * 9 x 1.60219 eV*A with the reference's qe = 1.60219e-19 and eV = 1.60219e-12 erg. */
static void hehe_nn(double r, double *potr, double *fpotr)
{
    if (r < 1.0) {
        const double ke = 9.0 * 1.60219 * 4.0;                       /* Z1 Z2 e^2 / (4 pi eps0) */
        const double as = 0.88534 * 0.5291772108 / (2.0 * pow(2.0, 0.23));
        double phi, mdphi;
        zbl_phi(r / as, &phi, &mdphi);
        const double v = ke * phi / r;
        *potr = 0.5 * v;
        *fpotr = v / r + ke * mdphi / (as * r);
    } else if (r < 1.3) {
        /* the cubic's CGS coefficients (:9-12) in eV, eV/A, eV/A^2, eV/A^3; the last two are
         * single-precision literals in the source (no exponent letter) */
        const double e = 1.60219e-12;
        const double c0 = 3.5443059983603055e-11 / e, c1 = -4.8619762395294636e-3 * 1e-8 / e;
        const double c2 = (double)(float)200609.6243721997 * 1e-16 / e;
        const double c3 = (double)(float)-2069784026620.333 * 1e-24 / e;
        *potr = 0.5 * (c0 + r * (c1 + r * (c2 + r * c3)));
        *fpotr = -(c1 + r * (2.0 * c2 + 3.0 * c3 * r));
    } else {
        const double ce = 0.000930644, r0 = 2.9673, al = 13.1;
        const double ex = exp(al * (1.0 - r / r0)), s6 = pow(r0 / r, 6.0);
        *potr = 0.5 * ce * (6.0 / (al - 6.0) * ex - al / (al - 6.0) * s6);
        *fpotr = ce * (6.0 * al / ((al - 6.0) * r0) * ex - 6.0 * al / (al - 6.0) * s6 / r);
    }
}

/* He-W, ZBL_ABINTIO_He_W_930.F90:58-176, in Angstrom / eV: ZBL with SI constants below
 * 1.5778 A (4 pi with the reference's pi = 3.141592654), six cubics to 3.5 A, then an EXP6 form
 * times the switch s = (1 - sin(pi (r - 5.8)/3))/2 on [4.3, 7.3] A whose derivative the
 * reference takes as -cos(pi (r - 5.8)/3)/2 (no factor pi/3), reproduced here. */
static void hew_nn(double r, double *potr, double *fpotr)
{
    static const double edge[7] = {1.57783601880074, 1.94810507446527, 2.10799896717072,
                                   2.22277348041534, 2.32289959788322, 3.05974050760269, 3.5};
    static const double c[6][4] = {
        {-54.6920134504158, 147.764553002780, -106.604073601512, 23.3457856042901},
        {8.13894099222489, -6.77821270976276, 2.38825082778931, -0.378954410552979},
        {11.8316959842284, -9.92672851472125, 2.88240909576416, -0.299054384231567},
        {18.5956897803305, -18.0913941109865, 6.12169742584229, -0.719758272171021},
        {11.5965650160971, -9.38901671011024, 2.52039670944214, -0.223789215087891},
        {11.0095425643702, -9.03994004997097, 2.48033046722412, -0.227488279342651}};
    if (r < edge[0]) {
        /* q Z1 Z2 / (4 pi eps0 r[m]) volts = eV per elementary charge; a in m */
        const double k = 1.60219e-19 * 2.0 * 74.0 / (4.0 * 3.141592654 * 8.854187817e-12) * 1e10;
        const double a = 0.88534 * 5.291772108e-11 / (pow(2.0, 0.23) + pow(74.0, 0.23)) * 1e10;
        double phi, mdphi;
        zbl_phi(r / a, &phi, &mdphi);
        *potr = 0.5 * k * phi / r;
        *fpotr = k * (phi / (r * r) + mdphi / (a * r));
        return;
    }
    if (r < 3.5) {
        int s = 5;
        for (int q = 0; q < 6; ++q)
            if (r < edge[q + 1]) { s = q; break; }
        *potr = 0.5 * (c[s][0] + r * (c[s][1] + r * (c[s][2] + r * c[s][3])));
        *fpotr = -(c[s][1] + r * (2.0 * c[s][2] + 3.0 * c[s][3] * r));
        return;
    }
    const double ea = 0.0084600, eb = 9.6004204435, ec = 4.135;
    double sw = 1.0, dsw = 0.0;
    if (r >= 7.3) { sw = 0.0; }
    else if (r > 4.3) {
        const double ph = 3.141592654 * (r - 5.8) / 3.0;
        sw = 0.5 * (1.0 - sin(ph));
        dsw = -0.5 * cos(ph);
    }
    const double ex = 6.0 / (eb - 6.0) * exp(eb * (1.0 - r / ec));
    const double v = ea * (ex - eb / (eb - 6.0) * pow(ec / r, 6.0));
    const double mdv = ea * (ex * eb / ec - 6.0 * eb / (eb - 6.0) * pow(ec / r, 6.0) / r);
    *potr = 0.5 * v * sw;
    *fpotr = mdv * sw - v * dsw;
}

static void zero_ne(double r, double *potb, double *fpotb)
{
    (void)r;
    *potb = 0.0;
    *fpotb = 0.0;
}

/* Bonny, Grigorev, Terentyev W-H-He EAM (EAM1_WHeH_Bonny_JPCM26_2014.F90), Angstrom / eV.
 * Knot sums V = sum a_k (r_k - r)^3 for r <= r_k (NN_FuncPoly3, MD_Pot_EAM_Utilities.F90:48-85). */
typedef struct { int n; double a[4], k[4]; } knots_t;

static void knot_pair(const knots_t *p, double r, double *potr, double *fpotr)
{
    double v = 0.0, d = 0.0;
    for (int i = 0; i < p->n; ++i) {
        const double x = p->k[i] - r;
        if (x < 0.0) continue;
        v += p->a[i] * x * x * x;
        d += p->a[i] * x * x;
    }
    *potr = 0.5 * v;
    *fpotr = 3.0 * d;
}

/* table t (1-based, registration order) of subtype sub (1 = EAM1, 2 = EAM2):
 * (W,W) (H,W) (He,W) (W,H) (H,H) (He,H) (W,He) (H,He) (He,He) [+ a zero #10 for EAM2] as
 * (source, target); returns -1 for an unknown table */
int orc_bonny_pair(int sub, int t, double r, double *potr, double *fpotr, double *potb, double *fpotb)
{
    static const knots_t k1[5] = {                        /* WH, WHe, HH, HHe, HeHe of EAM1 */
        {2, {13.75733214, 0.1296071475}, {2.0, 3.0}},
        {3, {21.0, 0.8565323293, 0.2750099819}, {1.9, 2.2, 3.5}},
        {2, {0.4862785907, 0.1018797872}, {2.0, 3.0}},
        {3, {15.0, 0.2563700119, -0.04489510592}, {1.8, 2.0, 3.0}},
        {2, {2.106615791, -0.2217639348}, {2.0, 3.0}}};
    static const knots_t k2[5] = {                        /* the same for EAM2 */
        {3, {44.24459079, -4.993477782, 1.461712984}, {2.0, 2.6475, 3.295}},
        {4, {0.0, 14.0, -3.712116187, 0.3105031456}, {1.9, 2.0, 2.2, 3.5}},
        {4, {40.0, 0.2315124670, -0.2, 0.05180584543}, {1.6, 2.0, 2.2, 3.0}},
        {3, {3.256370012, -0.4, -0.04489510592}, {2.0, 2.5, 3.0}},
        {4, {20.0, 1.051327582, -4.0, 0.03203322671}, {1.8, 2.0, 2.1, 3.0}}};
    static const int fn[10] = {-1, 0, 1, 0, 2, 3, 1, 3, 4, -2};
    const double gc = 1.848055990, gs = 2.232322602e-1;
    if (t < 1 || t > (sub == 2 ? 10 : 9)) return -1;
    *potr = *fpotr = *potb = *fpotb = 0.0;
    const int f = fn[t - 1];
    if (f == -2) return 0;
    double rho = 0.0, mdrho = 0.0;
    if (f == -1 || (sub == 2 && t == 4)) {               /* the gauge-transformed Marinica density */
        mar_ne(r, &rho, &mdrho);
        *potb = gs * rho;
        *fpotb = gs * mdrho;
    }
    if (f == -1) {                                       /* W-W: Marinica pair minus 2C rho */
        double v2, mdv;
        mar_nn(r, &v2, &mdv);
        *potr = v2 - gc * rho;
        *fpotr = mdv - 2.0 * gc * mdrho;
    } else {
        knot_pair(sub == 2 ? &k2[f] : &k1[f], r, potr, fpotr);
    }
    return 0;
}

/* embedding of group g (1 W, 2 H, 3 He): W the gauge-transformed Marinica F below
 * rho_I = 1.359141225 and a cubic above; H (EAM2 only) -26.10066441 sqrt(rho) + 0.4688963869 rho^2 */
int orc_bonny_embed(int sub, int g, double rho, double *f, double *df)
{
    *f = *df = 0.0;
    if (g == 1) {
        const double gc = 1.848055990, gs = 2.232322602e-1;
        if (rho <= 1.359141225) {
            double tf, tdf;
            const double tr = rho * (1.0 / gs);
            mar_embed(tr, &tf, &tdf);
            *f = tf + gc * tr;
            *df = tdf * (1.0 / gs) + gc * (1.0 / gs);
        } else {
            const double c[4] = {-5.524855802, 2.317313103e-1, -3.665345949e-2, 8.989367404e-3};
            *f = c[0] + c[1] * rho + c[2] * rho * rho + c[3] * rho * rho * rho;
            *df = c[1] + 2.0 * c[2] * rho + 3.0 * c[3] * rho * rho;
        }
        return 0;
    }
    if (g == 2 && sub == 2 && rho > 0.0) {
        *f = -26.10066441 * sqrt(rho) + 0.4688963869 * rho * rho;
        *df = -13.050332205 / sqrt(rho) + 2.0 * 0.4688963869 * rho;
    }
    return 0;
}

/* Ackland-Vitek Cu, Au, Cu-Au (EM_TB_{CuCu,AuAu,CuAu}_Ackland_Vitek_PRB41_10324.F90), FS form,
 * restated in Angstrom / eV.  Source literals without a D exponent are single precision
 * (float literals here).  The Cu-Au density derivative of the reference (:180-197) is
 * 1.5 sum A A (X+Y) (XY)^2 in its CGS units, i.e. 1.5 EVERG^2 sum A A (X+Y) (XY)^2 in eV / A
 * with A in eV^2/A^3; reproduced as such. */
typedef struct {
    double ar[6], rcr[6], at[2], rct[2], r11, r21, as, zz, c[4];
} av_t;

static av_t av_params(int which)
{
    const double ev = 1.60219e-12;
    av_t p;
    memset(&p, 0, sizeof(p));
    if (which == 0) {
        const double rr = 3.615;
        const float a[6] = {61.73525861f, -108.1846780f, 57.00053948f, -12.88796578f, 39.163819010f, 0.0f};
        const float m[6] = {1.225f, 1.202f, 1.154f, 1.050f, 0.866f, 0.707f};
        for (int k = 0; k < 6; ++k) { p.ar[k] = 0.5 * a[k] / (rr * rr * rr); p.rcr[k] = m[k] * rr; }
        p.at[0] = 10.03718305f / (rr * rr * rr); p.rct[0] = 1.225f * rr;
        p.at[1] = 17.06363299f / (rr * rr * rr); p.rct[1] = 0.990f * rr;
        p.r11 = 1.65; p.r21 = 1.90; p.as = 0.0738f; p.zz = 29.0 * 29.0;
        p.c[0] = 0.825015e-09; p.c[1] = -0.130825; p.c[2] = 0.696400e+07; p.c[3] = -0.124069e+15;
    } else if (which == 1) {
        const double rr = 4.078;
        const float a[6] = {29.059066f, -153.14779f, 148.17881f, -22.20508f, 72.71465f, 199.26269f};
        const float m[6] = {1.2247449f, 1.1547054f, 1.1180065f, 1.0000000f, 0.8660254f, 0.7071068f};
        for (int k = 0; k < 6; ++k) { p.ar[k] = 0.5 * a[k] / (rr * rr * rr); p.rcr[k] = m[k] * rr; }
        p.at[0] = 21.930125f / (rr * rr * rr); p.rct[0] = 1.1180065f * rr;
        p.at[1] = 284.99631f / (rr * rr * rr); p.rct[1] = 0.8660254f * rr;
        p.r11 = 1.85; p.r21 = 2.10; p.as = 0.0752; p.zz = 79.0 * 79.0;
        p.c[0] = 0.333482e-08; p.c[1] = -0.476248; p.c[2] = 0.228187e+08; p.c[3] = -0.365939e+15;
    } else {
        p.ar[0] = -0.0855455166 * 0.5; p.rcr[0] = 4.3098160;
        p.ar[1] = 0.1928358800 * 0.5;  p.rcr[1] = 4.0474790;
        p.ar[2] = 0.7593228600 * 0.5;  p.rcr[2] = 3.2979464;
        p.r11 = 1.85; p.r21 = 2.05; p.as = 0.0745; p.zz = 29.0 * 79.0;
        p.c[0] = 0.172724e-08; p.c[1] = -0.253573; p.c[2] = 0.124675e+08; p.c[3] = -0.204896e+15;
    }
    /* the cubic bridge's CGS coefficients in eV, eV/A, eV/A^2, eV/A^3 */
    p.c[0] /= ev; p.c[1] *= 1e-8 / ev; p.c[2] *= 1e-16 / ev; p.c[3] *= 1e-24 / ev;
    return p;
}

static void av_nn(int which, double r, double *potr, double *fpotr)
{
    const av_t p = av_params(which);
    if (r < p.r11) {
        /* Moliere: k e^2 with k = 9e9, e = 1.6029e-19 C (the source's values), in eV*A */
        const double ke2 = 9.0e9 * 1.6029e-19 * 1.6029e-19 * 1e9 / 1.60219e-12 * 1e8 * p.zz;
        const double x = r / p.as;
        const double s = 0.35 * exp(-0.3 * x) + 0.55 * exp(-1.2 * x) + 0.1 * exp(-6.0 * x);
        const double ds = 0.35 * (double)0.3f * exp(-0.3 * x) + 0.55 * 1.2 * exp(-1.2 * x) + 0.1 * 6.0 * exp(-6.0 * x);
        *potr = 0.5 * ke2 * s / r;
        *fpotr = ke2 * s / (r * r) + ke2 * ds / (r * p.as);
    } else if (r < p.r21) {
        *potr = 0.5 * (p.c[0] + r * (p.c[1] + r * (p.c[2] + r * p.c[3])));
        *fpotr = -(p.c[1] + r * (2.0 * p.c[2] + 3.0 * p.c[3] * r));
    } else {
        double v = 0.0, d = 0.0;
        for (int k = 0; k < 6; ++k) {
            if (!(r < p.rcr[k])) continue;
            const double t = p.rcr[k] - r;
            v += p.ar[k] * t * t * t;
            d += 6.0 * p.ar[k] * t * t;
        }
        *potr = v;
        *fpotr = d;
    }
}

static void av_ne(int which, double r, double *potb, double *fpotb)
{
    *potb = *fpotb = 0.0;
    if (which < 2) {
        const av_t p = av_params(which);
        for (int k = 0; k < 2; ++k) {
            if (!(r > 0.0 && r < p.rct[k])) continue;
            const double t = p.rct[k] - r;
            *potb += p.at[k] * t * t * t;
            *fpotb += 3.0 * p.at[k] * t * t;
        }
        return;
    }
    const av_t cu = av_params(0), au = av_params(1);
    const double xc[2] = {cu.rct[0] - r, cu.rct[1] - r}, xa[2] = {au.rct[0] - r, au.rct[1] - r};
    double q = 0.0, dq = 0.0;
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c) {
            if (!(r > 0.0 && xa[a] > 0.0 && xc[c] > 0.0)) continue;
            const double pr = xa[a] * xc[c];
            q += au.at[a] * cu.at[c] * pr * pr * pr;
            dq += 1.5 * au.at[a] * cu.at[c] * (xa[a] + xc[c]) * pr * pr;
        }
    if (r >= cu.rct[0]) { q = 0.0; dq = 0.0; }    /* no branch of the source beyond Cu's RCT1 */
    *potb = sqrt(q);
    *fpotb = dq * 1.60219e-12 * 1.60219e-12;
}

/* Mendelev-Ackland Zr EAM, EAM_ZrZr_Mendelev_Phil_Mag_L87_2007.F90:18-150 (Angstrom / eV in the
 * source itself).  Float literals: the source's default-REAL constants (0.1818, 0.5099, 0.2802,
 * 0.02817, 2.3000, 5.6, 7.6).  Step functions: [x >= 0] and, at 1 A and 2.3 A upper ends, [x > 0]. */
static double zr_knots(const double *c, double k, double r, double *mdv)
{
    double v = 0.0, d = 0.0;
    if (k - r >= 0.0)
        for (int n = 4; n <= 8; ++n) {
            v += c[n - 4] * pow(k - r, (double)n);
            d += c[n - 4] * n * pow(k - r, (double)(n - 1));
        }
    *mdv = d;
    return v;
}

static void zr_nn(double r, double *potr, double *fpotr)
{
    static const double c35[5] = {-1.4261501929757e+01, 1.5850036758176e+01, -1.1325102264291e+01,
                                  -4.0971114831366e+00, 3.6739378016909e+00};
    static const double c60[5] = {1.3066813393823e+00, -6.0542710718094e-01, 1.0055527194350e+00,
                                  -1.4918186777562e-01, 3.2773112059590e-02};
    static const double c76[5] = {1.1433120304691e-02, -2.1982172508973e-02, -1.2542439692607e-02,
                                  2.5062673874258e-02, -7.5442887837418e-03};
    const double r23 = 2.3000f;
    double v = 0.0, d = 0.0;
    if (1.0 - r > 0.0) {
        const double q = 2.3039613229091e+04;
        const double t1 = 0.1818f * exp(-3.3035595072498e+01 * r), t2 = 0.5099f * exp(-9.7279503865046e+00 * r);
        const double t3 = 0.2802f * exp(-4.1593878920967e+00 * r), t4 = 0.02817f * exp(-2.0812424895674e+00 * r);
        v += q / r * (t1 + t2 + t3 + t4);
        d += q / r * ((1.0 / r + 3.3035595072498e+01) * t1 + (1.0 / r + 9.7279503865046e+00) * t2 +
                      (1.0 / r + 4.1593878920967e+00) * t3 + (1.0 / r + 2.0812424895674e+00) * t4);
    }
    if (r - 1.0 >= 0.0 && r23 - r > 0.0) {
        const double pe = 1.2333392307614e+01 - 1.0847321969086e+01 * r + 4.5733524424508e+00 * r * r -
                          8.5266291445935e-01 * r * r * r;
        v += exp(pe);
        d -= (-1.0847321969086e+01 + 9.1467048849017e+00 * r - 2.5579887433781e+00 * r * r) * exp(pe);
    }
    if (r - r23 >= 0.0) {
        double d1, d2, d3;
        v += zr_knots(c35, 3.5, r, &d1) + zr_knots(c60, 6.0, r, &d2) + zr_knots(c76, (double)7.6f, r, &d3);
        d += d1 + d2 + d3;
    }
    *potr = 0.5 * v;
    *fpotr = d;
}

static void zr_ne(double r, double *potb, double *fpotb)
{
    static const double cr[5] = {7.7718711248373e-01, -4.8102928454986e-01, 1.4501312593993e-01,
                                 -2.1292226813959e-02, 1.2209217625670e-03};
    *potb = zr_knots(cr, (double)5.6f, r, fpotb);
}

static void zr_embed(double rho, double *f, double *df)
{
    static const double rk[5] = {60.0, 70.0, 80.0, 85.0, 90.0};
    static const double ck[5] = {-1.9162462126235e-07, 4.6418727035037e-07, 6.6448294272955e-07,
                                 -2.0680252960229e-06, 1.1387131464983e-06};
    *f = -pow(rho, 0.5);
    *df = -0.5 / pow(rho, 0.5);                 /* -inf at rho = 0, as in the reference */
    for (int k = 0; k < 5; ++k) {
        if (rho - rk[k] < 0.0) continue;
        *f += ck[k] * pow(rho - rk[k], 4.0);
        *df += 4.0 * ck[k] * pow(rho - rk[k], 3.0);
    }
}

/* Ackland-Wooding-Bacon Zr, EM_TB_AWB_Phil_Mag_A71_1995_553.F90 (FS form), Angstrom / eV.  Scale
 * length s = 3.249 A * 1.414213562 (CP_RSQ2); float literals for the source's default-REAL
 * constants; zero beyond the last knot (the source leaves those zero-initialised entries). */
static void awb_nn(double r, double *potr, double *fpotr)
{
    const double ev = 1.60219e-12, s = 3.249 * 1.414213562;
    static const float ar[7] = {-58.480671f, 83.692945f, -20.958026f, -1.309533f, 65.726356f, 139.411255f,
                                443.442749f};
    static const float mr[7] = {1.22f, 1.20f, 1.14f, 0.95f, 0.80f, 0.70f, 0.63f};
    if (r < 1.20) {
        /* ZBL with Z1 = Z2 = 40: 9e9 qe^2 = 9 x 1.60219 eV*A (qe = 1.60219e-19, eV = qe 1e7 erg) */
        const double ke = 9.0 * 1.60219 * 1600.0;
        const double as = 0.88534 * 0.5291772108 / (2.0 * pow(40.0, 0.23));
        double phi, mdphi;
        zbl_phi(r / as, &phi, &mdphi);
        *potr = 0.5 * ke * phi / r;
        *fpotr = ke * phi / (r * r) + ke * mdphi / (as * r);
    } else if (r <= 2.55) {
        const double q = exp(13.4037f + r * (-12.2190f + r * (5.0261f + r * -0.8435f)));
        *potr = 0.5 * q;
        *fpotr = -(-12.2190f + 2.0 * 5.0261f * r + 3.0 * -0.8435f * r * r) * q;
    } else if (r <= mr[6] * s) {
        /* cubic with CGS coefficients: eV, eV/A, eV/A^2, eV/A^3 after conversion */
        const double c0 = 5.0256487041006336e-010 / ev, c1 = -5.0454065151782766e-002 * 1e-8 / ev;
        const double c2 = 1706444.034874689 * 1e-16 / ev, c3 = -19388949878932.86 * 1e-24 / ev;
        *potr = 0.5 * (c0 + r * (c1 + r * (c2 + r * c3)));
        *fpotr = -(c1 + r * (2.0 * c2 + 3.0 * c3 * r));
    } else {
        double v = 0.0, d = 0.0;
        for (int k = 0; k < 7; ++k) {
            const double kk = mr[k] * s;
            if (!(r < kk)) continue;
            v += ar[k] / (s * s * s) * pow(kk - r, 3.0);
            d += 3.0 * ar[k] / (s * s * s) * pow(kk - r, 2.0);
        }
        *potr = 0.5 * v;
        *fpotr = d;
    }
}

static void awb_ne(double r, double *potb, double *fpotb)
{
    const double s = 3.249 * 1.414213562;
    const double k1 = 1.22f * s, k2 = 1.05f * s, a1 = 48.288836f / (s * s * s), a2 = -0.850556f / (s * s * s);
    *potb = *fpotb = 0.0;
    if (r > 0.0 && r < k1) {
        *potb = a1 * pow(k1 - r, 3.0);
        *fpotb = 3.0 * a1 * pow(k1 - r, 2.0);
        if (r < k2) {
            *potb += a2 * pow(k2 - r, 3.0);
            *fpotb += 3.0 * a2 * pow(k2 - r, 2.0);
        }
    }
}

/* He-Ti, EM_TB_WangJun_Ti-HE_2007/LJ_He_Ti.F90:10-28, Angstrom / eV: phi0 = 0.02617 eV,
 * r0 = 4.72879 A; the exponents 4.35 and 1.4 are single-precision literals in the source, the
 * derivative's factors double. */
static void heti_nn(double r, double *potr, double *fpotr)
{
    const double phi0 = 0.02617, r0 = 4.72879;
    const double a = pow(r0 / r, (double)4.35f), b = pow(r0 / r, (double)1.4f);
    *potr = 0.5 * phi0 * (a - 3.211829 * b);
    *fpotr = phi0 * (4.35 * a - 3.211829 * 1.4 * b) / r;
}

int orc_pot_eval(int pot, const double *prm, double r, double *potr, double *fpotr,
                 double *potb, double *fpotb)
{
    switch (pot) {
    case ORC_POT_CR: cr_nn(r, prm, potr, fpotr); cr_ne(r, prm, potb, fpotb); return 0;
    case ORC_POT_MARINICA2: mar_nn(r, potr, fpotr); mar_ne(r, potb, fpotb); return 0;
    case ORC_POT_AV_CU: av_nn(0, r, potr, fpotr); av_ne(0, r, potb, fpotb); return 0;
    case ORC_POT_AV_AU: av_nn(1, r, potr, fpotr); av_ne(1, r, potb, fpotb); return 0;
    case ORC_POT_AV_CUAU: av_nn(2, r, potr, fpotr); av_ne(2, r, potb, fpotb); return 0;
    case ORC_POT_MENDELEV_ZR: zr_nn(r, potr, fpotr); zr_ne(r, potb, fpotb); return 0;
    case ORC_POT_AWB_ZR: awb_nn(r, potr, fpotr); awb_ne(r, potb, fpotb); return 0;
    case ORC_POT_HETI_LJ: heti_nn(r, potr, fpotr); zero_ne(r, potb, fpotb); return 0;
    case ORC_POT_MARINICA3:
    case ORC_POT_MARINICA4: {
        const mar_set_t *m = &mar_sets[pot == ORC_POT_MARINICA3 ? 1 : 2];
        mar_set_nn(m, r, potr, fpotr);
        mar_set_ne(m, r, potb, fpotb);
        return 0;
    }
    case ORC_POT_ACKLAND_WW: ack_nn(r, potr, fpotr); ack_ne(r, potb, fpotb); return 0;
    case ORC_POT_DERLET_WW: der_nn(r, potr, fpotr); der_ne(r, potb, fpotb); return 0;
    case ORC_POT_HEHE_EXP6: hehe_nn(r, potr, fpotr); zero_ne(r, potb, fpotb); return 0;
    case ORC_POT_HEW_ZBL: hew_nn(r, potr, fpotr); zero_ne(r, potb, fpotb); return 0;
    default: return -1;
    }
}

int orc_embed_eval(int pot, const double *prm, double rho, double *f, double *df)
{
    (void)prm;
    if (pot == ORC_POT_MARINICA2) { mar_embed(rho, f, df); return 0; }
    if (pot == ORC_POT_MARINICA3) { mar_set_embed(&mar_sets[1], rho, f, df); return 0; }
    if (pot == ORC_POT_MARINICA4) { mar_set_embed(&mar_sets[2], rho, f, df); return 0; }
    if (pot == ORC_POT_MENDELEV_ZR) { zr_embed(rho, f, df); return 0; }
    *f = 0.0; *df = 0.0;
    return -1;
}

/* Create_Pairwise_ForceTable (MD_TypeDef_ForceTable.F90:949-976) and Create_EMBDFUNTable
 * (:1040-1048) for one species:  T = i*CSIV, R = T*T;  POTR = f1(R)*R, FPOTR = f2(R)*R,
 * POTB = rho(R), FPOTB = -rho'(R);  RHOMX = RHOSCAL * max POTB;  RHOD = RHOMX / NEMBD;
 * F and F' tabulated at rho = (i-1)*RHOD. */
int orc_make_tables(int pot, const double *prm, double rmax, int ntab, int nembd, double rhoscal,
                    double *potr, double *fpotr, double *potb, double *fpotb,
                    double *fembd, double *dfembd, double *rhod)
{
    double rmaxsqrt = sqrt(rmax);
    double csi = (double)ntab / rmaxsqrt;
    double csiv = 1.0 / csi;
    double rhomx = -1.0;
    for (int i = 1; i <= ntab; ++i) {
        double t = (double)i * csiv;
        double r = t * t;
        double a, b, c, d;
        if (orc_pot_eval(pot, prm, r, &a, &b, &c, &d) != 0) return -1;
        potr[i - 1] = a * r;
        fpotr[i - 1] = b * r;
        potb[i - 1] = c;
        fpotb[i - 1] = d;
        if (rhomx < c * rhoscal) rhomx = c * rhoscal;
    }
    double rd = rhomx / (double)nembd;
    if (rhod) *rhod = rd;
    if (fembd && dfembd) {
        for (int i = 1; i <= nembd; ++i) {
            double rho = (double)(i - 1) * rd;
            if (orc_embed_eval(pot, prm, rho, &fembd[i - 1], &dfembd[i - 1]) != 0) {
                fembd[i - 1] = 0.0;
                dfembd[i - 1] = 0.0;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* table lookups                                                                         */
/* ------------------------------------------------------------------------------------ */

static inline double tab(const double *T, int nkind, int ntab, int k, int i)
{
    if (i < 1) return 0.0;          /* padding: never reached for r > CSIV^2 */
    if (i > ntab) i = ntab;         /* padding: r == Rmax exactly reads NTAB+1 with DK = 0 */
    return T[(size_t)(i - 1) * (size_t)nkind + (size_t)k];
}

/* linear interpolation in the sqrt(r) grid: T(KK) + DK (T(KK+1) - T(KK)) */
static inline double interp(const double *T, int nkind, int ntab, int k, int kk, double dk)
{
    double a = tab(T, nkind, ntab, k, kk);
    double b = tab(T, nkind, ntab, k, kk + 1);
    return a + dk * (b - a);
}

static inline double slope(const double *T, int nkind, int ntab, int k, int kk)
{
    return tab(T, nkind, ntab, k, kk + 1) - tab(T, nkind, ntab, k, kk);
}

/* non-cubic box: DXYZ(K) = sum(BOXSHAPE(K,1:3)*SEP(1:3)), MD_FS_ForceTable.F90:235,333 and
   MD_NeighborsList.F90:362-364 (the Fortran sum adds left to right) */
static inline void shape_sep(const orc_box *b, double *sx, double *sy, double *sz)
{
    if (!b->shaped) return;
    const double x = *sx, y = *sy, z = *sz;
    *sx = b->bs[0] * x + b->bs[1] * y + b->bs[2] * z;
    *sy = b->bs[3] * x + b->bs[4] * y + b->bs[5] * z;
    *sz = b->bs[6] * x + b->bs[7] * y + b->bs[8] * z;
}

/* minimum image, MD_FS_ForceTable_GPU.F90:464-476 */
static inline double min_image(double s, double len, double half, int pd)
{
    if (pd && fabs(s) > half) s = s - copysign(len, s);
    return s;
}

/* ------------------------------------------------------------------------------------ */
/* neighbour list, Cal_NeighboreList2C (MD_NeighborsList.F90:396-633)                   */
/* ------------------------------------------------------------------------------------ */

static const int NIX[27] = {0, -1, -1, -1, 0, 0, -1, 1, -1, 0, 1, -1, 0, 1, 1, 1, 1, 0, 0, -1, 1, -1, 0, 1, -1, 0, 1};
static const int NIY[27] = {0, 0, -1, 1, 1, 0, 0, 0, -1, -1, -1, 1, 1, 1, 0, 1, -1, -1, 0, 0, 0, -1, -1, -1, 1, 1, 1};
static const int NIZ[27] = {0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, -1};

int orc_nlist(int n, const double *x, const double *y, const double *z, const int *statu,
              const orc_box *box, double rc_nl, int mxkvois, int *kvois, int *indi, int *ncell3)
{
    const double eps = 0.0001;
    int nc[3];
    if (box->shaped) {   /* cells of rc_nl in box units need not cover rc_nl after the shape */
        if (ncell3) ncell3[0] = ncell3[1] = ncell3[2] = 0;
        return orc_nlist_brute(n, x, y, z, statu, box, rc_nl, mxkvois, kvois, indi);
    }
    for (int k = 0; k < 3; ++k) {
        nc[k] = (int)(box->len[k] / (1.0 * rc_nl) - eps);   /* :476 */
        if (nc[k] < 3) nc[k] = 3;                            /* :478, C_ITHR */
    }
    if (ncell3) { ncell3[0] = nc[0]; ncell3[1] = nc[1]; ncell3[2] = nc[2]; }
    const int ncell = nc[0] * nc[1] * nc[2];
    int *head = (int *)malloc(sizeof(int) * (size_t)ncell);
    int *link = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *cellof = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int c = 0; c < ncell; ++c) head[c] = -1;
    const double *xp[3] = {x, y, z};
    const double rc2 = rc_nl * rc_nl;
    const double half[3] = {0.5 * box->len[0], 0.5 * box->len[1], 0.5 * box->len[2]};
    int err = 0;

    /* linked cells, head insertion (:497-530) */
    for (int i = 0; i < n; ++i) {
        kvois[i] = 0;
        cellof[i] = -1;
        if (statu[i] & ORC_STATU_OUTOFBOX) continue;
        int ixyz[3];
        for (int k = 0; k < 3; ++k) {
            ixyz[k] = (int)((xp[k][i] - box->lo[k]) / box->len[k] * (double)nc[k] - eps);
            if (ixyz[k] < 0 || ixyz[k] > nc[k]) err = -2;
            if (ixyz[k] >= nc[k]) ixyz[k] = nc[k] - 1;
            if (ixyz[k] < 0) ixyz[k] = 0;
        }
        int ic = ixyz[0] + nc[0] * (ixyz[1] + nc[1] * ixyz[2]);
        cellof[i] = ic;
        link[i] = head[ic];
        head[ic] = i;
    }
    if (err) { free(head); free(link); free(cellof); return err; }

    int overflow = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : overflow)
    for (int c = 0; c < ncell; ++c) {
        if (head[c] < 0) continue;
        int iz = c / (nc[0] * nc[1]);
        int iy = (c / nc[0]) % nc[1];
        int ix = c % nc[0];
        /* candidates: own cell first, then the stencil NIX/NIY/NIZ(2..27) (:540-585) */
        int cap = 1024, ncand = 0, n0 = 0;
        int *cand = (int *)malloc(sizeof(int) * (size_t)cap);
        for (int s = 0; s < 27; ++s) {
            int j3[3] = {ix + NIX[s], iy + NIY[s], iz + NIZ[s]};
            int skip = 0;
            for (int k = 0; k < 3; ++k) {
                if (box->ifpd[k]) {
                    if (j3[k] >= nc[k]) j3[k] = 0;
                    else if (j3[k] < 0) j3[k] = nc[k] - 1;
                }
                if (j3[k] < 0 || j3[k] >= nc[k]) skip = 1;
            }
            if (skip) continue;
            int jc = j3[0] + nc[0] * (j3[1] + nc[1] * j3[2]);
            for (int id = head[jc]; id >= 0; id = link[id]) {
                if (ncand == cap) { cap *= 2; cand = (int *)realloc(cand, sizeof(int) * (size_t)cap); }
                cand[ncand++] = id;
            }
            if (s == 0) n0 = ncand;
        }
        for (int a = 0; a < n0; ++a) {
            int i = cand[a];
            int nn = 0;
            for (int b = 0; b < ncand; ++b) {
                if (b == a) continue;
                int j = cand[b];
                double d2 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    double s = min_image(xp[k][i] - xp[k][j], box->len[k], half[k], box->ifpd[k]);
                    d2 += s * s;
                }
                if (d2 < rc2) {                             /* :605, strict */
                    if (nn >= mxkvois) { overflow = 1; break; }
                    indi[(size_t)nn * (size_t)n + (size_t)i] = j;
                    ++nn;
                }
            }
            kvois[i] = nn;
        }
        free(cand);
    }
    free(head); free(link); free(cellof);
    return overflow ? -1 : 0;
}

int orc_nlist_brute(int n, const double *x, const double *y, const double *z, const int *statu,
                    const orc_box *box, double rc_nl, int mxkvois, int *kvois, int *indi)
{
    const double *xp[3] = {x, y, z};
    const double rc2 = rc_nl * rc_nl;
    const double half[3] = {0.5 * box->len[0], 0.5 * box->len[1], 0.5 * box->len[2]};
    int overflow = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : overflow)
    for (int i = 0; i < n; ++i) {
        int nn = 0;
        if (!(statu[i] & ORC_STATU_OUTOFBOX)) {
            for (int j = 0; j < n; ++j) {
                if (j == i || (statu[j] & ORC_STATU_OUTOFBOX)) continue;
                double sv[3];
                for (int k = 0; k < 3; ++k)
                    sv[k] = min_image(xp[k][i] - xp[k][j], box->len[k], half[k], box->ifpd[k]);
                shape_sep(box, &sv[0], &sv[1], &sv[2]);
                const double d2 = sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2];
                if (d2 < rc2) {
                    if (nn >= mxkvois) { overflow = 1; break; }
                    indi[(size_t)nn * (size_t)n + (size_t)i] = j;
                    ++nn;
                }
            }
        }
        kvois[i] = nn;
    }
    return overflow ? -1 : 0;
}

/* ------------------------------------------------------------------------------------ */
/* force passes                                                                          */
/* ------------------------------------------------------------------------------------ */

/* embedding derivative lookup, MD_EAM_ForceTable_GPU.F90:535-541 */
static inline double embd_lookup(const double *T, int nkind1, int nembd, int ke, double rho,
                                 double rhod, int *bad, double *sl)
{
    double sk = rho / rhod + 1.0;
    int kk = (int)(sk + 0.000001);
    if (kk + 1 > nembd) *bad = 1;
    double a = tab(T, nkind1, nembd, ke, kk);
    double b = tab(T, nkind1, nembd, ke, kk + 1);
    if (sl) *sl = b - a;
    return a + (sk - kk) * (b - a);
}

int orc_force(int n, const double *x, const double *y, const double *z, const int *ityp,
              const int *statu, const orc_box *box, const int *kvois, const int *indi, int ldi,
              const orc_tables *t, double *den, double *fx, double *fy, double *fz,
              double *epot, double *vir9, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const double bx = box->len[0], by = box->len[1], bz = box->len[2];
    const double hbx = 0.5 * bx, hby = 0.5 * by, hbz = 0.5 * bz;
    const int px = box->ifpd[0], py = box->ifpd[1], pz = box->ifpd[2];
    const int nk = t->nkind, nt = t->ntab, ng = t->ngroup;
    double *dn = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *pv = vir9 ? (double *)calloc((size_t)(n > 0 ? n : 1) * 6, sizeof(double)) : NULL;
    int nbad = 0;

    /* pass 1: electron density and F'(rho), PRECALFOR_KERNEL */
#pragma omp parallel for schedule(static) reduction(+ : nbad)
    for (int ic = 0; ic < n; ++ic) {
        double den0 = 0.0, er0 = 0.0;
        int ityi = ityp[ic];
        if ((statu[ic] & ORC_STATU_ACTIVE) == ORC_STATU_ACTIVE) {
            double posx = x[ic], posy = y[ic], posz = z[ic];
            int iiw = kvois[ic];
            for (int iw = 0; iw < iiw; ++iw) {
                int j = indi[(size_t)iw * (size_t)ldi + (size_t)ic];
                double sepx = min_image(posx - x[j], bx, hbx, px);
                double sepy = min_image(posy - y[j], by, hby, py);
                double sepz = min_image(posz - z[j], bz, hbz, pz);
                shape_sep(box, &sepx, &sepy, &sepz);
                double r2 = sepx * sepx + sepy * sepy + sepz * sepz;
                if (r2 <= t->ru2) {
                    int ktab = t->kpair[(ityp[j] - 1) * ng + (ityi - 1)] - 1;
                    double r = sqrt(r2);
                    double sk = sqrt(r) * t->csi;
                    int kk = (int)sk;
                    double dk = sk - kk;
                    den0 = den0 + interp(t->potb, nk, nt, ktab, kk, dk);
                    if (epot) er0 = er0 + interp(t->potr, nk, nt, ktab, kk, dk) / r;
                }
            }
            double d = den0;
            if (t->pottype == ORC_FS) {
                if (den0 > 0.0) d = -0.5 / sqrt(den0);
                if (epot) epot[ic] = er0 - sqrt(den0);
            } else {
                int ke = t->kembd[ityi - 1] - 1, bad = 0;
                if (den0 > 0.0) d = embd_lookup(t->dfembd, t->nkind1, t->nembd, ke, den0, t->rhod, &bad, NULL);
                if (epot) epot[ic] = er0 + embd_lookup(t->fembd, t->nkind1, t->nembd, ke, den0, t->rhod, &bad, NULL);
                nbad += bad;
            }
            dn[ic] = d;
        } else {
            dn[ic] = 0.0;
            if (epot) epot[ic] = (t->pottype == ORC_FS) ? 0.0 : 0.0;
        }
    }
    if (den) memcpy(den, dn, sizeof(double) * (size_t)n);

    /* pass 2: forces and virial, CALFORCE_KERNEL / CALPTENSOR_KERNEL */
    if (fx || vir9) {
#pragma omp parallel for schedule(static)
        for (int ic = 0; ic < n; ++ic) {
            double fpx = 0.0, fpy = 0.0, fpz = 0.0;
            double p11 = 0, p12 = 0, p13 = 0, p22 = 0, p23 = 0, p33 = 0;
            int ityi = ityp[ic];
            if ((statu[ic] & ORC_STATU_ACTIVE) == ORC_STATU_ACTIVE) {
                double posx = x[ic], posy = y[ic], posz = z[ic];
                double denki = dn[ic];
                int iiw = kvois[ic];
                for (int iw = 0; iw < iiw; ++iw) {
                    int j = indi[(size_t)iw * (size_t)ldi + (size_t)ic];
                    double sepx = min_image(posx - x[j], bx, hbx, px);
                    double sepy = min_image(posy - y[j], by, hby, py);
                    double sepz = min_image(posz - z[j], bz, hbz, pz);
                    shape_sep(box, &sepx, &sepy, &sepz);
                    double r2 = sepx * sepx + sepy * sepy + sepz * sepz;
                    if (r2 <= t->ru2) {
                        int ityj = ityp[j];
                        int ktab = t->kpair[(ityj - 1) * ng + (ityi - 1)] - 1;
                        int ktab1 = t->kpair[(ityi - 1) * ng + (ityj - 1)] - 1;
                        double r = sqrt(r2);
                        double sk = sqrt(r) * t->csi;
                        int kk = (int)sk;
                        double dk = sk - kk;
                        double denkj = dn[j];
                        double fortot = interp(t->fpotr, nk, nt, ktab, kk, dk) / r2 +
                                        (interp(t->fpotb, nk, nt, ktab, kk, dk) * denki +
                                         interp(t->fpotb, nk, nt, ktab1, kk, dk) * denkj) / r;
                        fpx = fpx + fortot * sepx;
                        fpy = fpy + fortot * sepy;
                        fpz = fpz + fortot * sepz;
                        if (pv) {
                            double hf = fortot * 0.5;
                            p11 += sepx * sepx * hf; p12 += sepx * sepy * hf; p13 += sepx * sepz * hf;
                            p22 += sepy * sepy * hf; p23 += sepy * sepz * hf; p33 += sepz * sepz * hf;
                        }
                    }
                }
            }
            if (fx) { fx[ic] = fpx; fy[ic] = fpy; fz[ic] = fpz; }
            if (pv) {
                double *q = pv + (size_t)ic * 6;
                q[0] = p11; q[1] = p12; q[2] = p13; q[3] = p22; q[4] = p23; q[5] = p33;
            }
        }
    }
    if (vir9) {
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 6; ++c) s[c] += pv[(size_t)i * 6 + c];
        vir9[0] = s[0]; vir9[1] = s[1]; vir9[2] = s[2];
        vir9[3] = s[1]; vir9[4] = s[3]; vir9[5] = s[4];
        vir9[6] = s[2]; vir9[7] = s[4]; vir9[8] = s[5];
        free(pv);
    }
    free(dn);
    return nbad;
}

/* ------------------------------------------------------------------------------------ */
/* Swope velocity Verlet                                                                 */
/* ------------------------------------------------------------------------------------ */

void orc_predictor(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                   const double *fx, const double *fy, const double *fz, double *dx, double *dy,
                   double *dz, int *statu, const int *ityp, const double *cm, double h,
                   const orc_box *box)
{
    const double th = h, hs2 = th * 0.5, h2s2 = th * th * 0.5;
    double lb[3], ub[3];
    for (int k = 0; k < 3; ++k) { lb[k] = box->lo[k]; ub[k] = box->lo[k] + box->len[k]; }
    double *xp[3] = {x, y, z}, *vp[3] = {vx, vy, vz}, *dp[3] = {dx, dy, dz};
    const double *fp[3] = {fx, fy, fz};
    const int fixpos[3] = {ORC_STATU_FIXPOSX, ORC_STATU_FIXPOSY, ORC_STATU_FIXPOSZ};
    const int fixvel[3] = {ORC_STATU_FIXVELX, ORC_STATU_FIXVELY, ORC_STATU_FIXVELZ};
    for (int i = 0; i < n; ++i) {
        int stat = statu[i];
        if ((stat & ORC_STATU_ACTIVE) != ORC_STATU_ACTIVE) continue;
        double cm0 = cm[ityp[i] - 1];
        double xn[3];
        for (int k = 0; k < 3; ++k) {
            double a = fp[k][i] / cm0;
            double dis = th * vp[k][i] + h2s2 * a;
            if (stat & fixpos[k]) dis = 0.0;
            double xv = xp[k][i] + dis;
            if (box->ifpd[k]) {
                if (xv > ub[k]) { xv = xv - box->len[k]; stat |= ORC_STATU_PASSBOUND; }
                else if (xv < lb[k]) { xv = xv + box->len[k]; stat |= ORC_STATU_PASSBOUND; }
            }
            if (!(stat & fixvel[k]) && !(stat & fixpos[k])) vp[k][i] = vp[k][i] + hs2 * a;
            xp[k][i] = xv;
            xn[k] = xv;
            dp[k][i] = dp[k][i] + dis;
        }
        /* PASSBOUND stays local; only the out-of-box flags are stored (:372-378) */
        if (xn[0] > ub[0] || xn[1] > ub[1] || xn[2] > ub[2])
            statu[i] = ORC_STATU_OUTOFBOX | ORC_STATU_REFLECT;
        else if (xn[0] < lb[0] || xn[1] < lb[1] || xn[2] < lb[2])
            statu[i] = ORC_STATU_OUTOFBOX | ORC_STATU_TRANSMIT;
    }
}

void orc_corrector(int n, double *vx, double *vy, double *vz, const double *fx, const double *fy,
                   const double *fz, const int *statu, const int *ityp, const double *cm, double h)
{
    const double hs2 = h * 0.5;
    for (int i = 0; i < n; ++i) {
        int stat = statu[i];
        if ((stat & ORC_STATU_ACTIVE) != ORC_STATU_ACTIVE) continue;
        double cm0 = cm[ityp[i] - 1];
        if (!(stat & ORC_STATU_FIXVELX) && !(stat & ORC_STATU_FIXPOSX)) vx[i] = vx[i] + hs2 * (fx[i] / cm0);
        if (!(stat & ORC_STATU_FIXVELY) && !(stat & ORC_STATU_FIXPOSY)) vy[i] = vy[i] + hs2 * (fy[i] / cm0);
        if (!(stat & ORC_STATU_FIXVELZ) && !(stat & ORC_STATU_FIXPOSZ)) vz[i] = vz[i] + hs2 * (fz[i] / cm0);
    }
}

/* external force fext (3n, x block then y then z; may be NULL) added to every active atom
 * after each force evaluation, as Calforce_ForceClass0 runs Cumulate_ExtForce0 after pCalForce
 * (MD_ForceClass_Register_GPU.F90:584-606, 636-656) */
static void add_ext(int n, const double *fext, const int *statu, double *fx, double *fy, double *fz)
{
    if (!fext) return;
    for (int i = 0; i < n; ++i) {
        if ((statu[i] & 1) != 1) continue;
        fx[i] += fext[i];
        fy[i] += fext[n + i];
        fz[i] += fext[2 * n + i];
    }
}

int orc_md(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
           double *fx, double *fy, double *fz, int *statu, const int *ityp, const orc_box *box,
           const orc_tables *t, const double *cm, double h, int nsteps, double rc_nl,
           double skin_trigger, int nb_uptab, int mxkvois, int nthreads)
{
    return orc_md_ext(n, x, y, z, vx, vy, vz, fx, fy, fz, statu, ityp, box, t, cm, h, nsteps, rc_nl,
                      skin_trigger, nb_uptab, mxkvois, nthreads, NULL);
}

int orc_md_ext(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
               double *fx, double *fy, double *fz, int *statu, const int *ityp, const orc_box *box,
               const orc_tables *t, const double *cm, double h, int nsteps, double rc_nl,
               double skin_trigger, int nb_uptab, int mxkvois, int nthreads, const double *fext)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    size_t nn = (size_t)(n > 0 ? n : 1);
    int *kvois = (int *)malloc(sizeof(int) * nn);
    int *indi = (int *)malloc(sizeof(int) * nn * (size_t)mxkvois);
    double *dsb = (double *)calloc(nn * 3, sizeof(double));
    int rebuilds = 0, rc;
    rc = orc_nlist(n, x, y, z, statu, box, rc_nl, mxkvois, kvois, indi, NULL);
    if (rc) goto done;
    orc_force(n, x, y, z, ityp, statu, box, kvois, indi, n, t, NULL, fx, fy, fz, NULL, NULL, nthreads);
    add_ext(n, fext, statu, fx, fy, fz);
    for (int step = 1; step <= nsteps; ++step) {
        orc_predictor(n, x, y, z, vx, vy, vz, fx, fy, fz, dsb, dsb + nn, dsb + 2 * nn, statu, ityp, cm, h, box);
        int rebuild = 0;
        if (skin_trigger > 0.0) {
            double mx = 0.0;
            for (int i = 0; i < n; ++i) {
                double d2 = dsb[i] * dsb[i] + dsb[nn + i] * dsb[nn + i] + dsb[2 * nn + i] * dsb[2 * nn + i];
                if (d2 > mx) mx = d2;
            }
            rebuild = mx > skin_trigger * skin_trigger;
        } else if (nb_uptab > 0) {
            rebuild = (step % nb_uptab) == 0;
        }
        if (rebuild) {
            rc = orc_nlist(n, x, y, z, statu, box, rc_nl, mxkvois, kvois, indi, NULL);
            if (rc) goto done;
            memset(dsb, 0, sizeof(double) * nn * 3);
            ++rebuilds;
        }
        orc_force(n, x, y, z, ityp, statu, box, kvois, indi, n, t, NULL, fx, fy, fz, NULL, NULL, nthreads);
        add_ext(n, fext, statu, fx, fy, fz);
        orc_corrector(n, vx, vy, vz, fx, fy, fz, statu, ityp, cm, h);
    }
    rc = rebuilds;
done:
    free(kvois); free(indi); free(dsb);
    return rc;
}

/* ------------------------------------------------------------------------------------ */
/* Per-atom virial tensor (MD_FS_ForceTable_GPU.F90:1746-1965; EAM :1775-1994)           */
/* ------------------------------------------------------------------------------------ */
void orc_atomic_stress(int n, const double *x, const double *y, const double *z, const int *ityp,
                       const int *statu, const orc_box *box, const int *kvois, const int *indi,
                       int ldi, const orc_tables *t, const double *den, double *ap, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const double bx = box->len[0], by = box->len[1], bz = box->len[2];
    const int px = box->ifpd[0], py = box->ifpd[1], pz = box->ifpd[2];
    const int nk = t->nkind, nt = t->ntab, ng = t->ngroup;
#pragma omp parallel for schedule(static)
    for (int ic = 0; ic < n; ++ic) {
        double p[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if ((statu[ic] & ORC_STATU_ACTIVE) == ORC_STATU_ACTIVE) {
            const int ityi = ityp[ic];
            const double denki = den[ic];
            for (int iw = 0; iw < kvois[ic]; ++iw) {
                int j = indi[(size_t)iw * (size_t)ldi + (size_t)ic];
                double s[3];
                s[0] = min_image(x[ic] - x[j], bx, 0.5 * bx, px);
                s[1] = min_image(y[ic] - y[j], by, 0.5 * by, py);
                s[2] = min_image(z[ic] - z[j], bz, 0.5 * bz, pz);
                shape_sep(box, &s[0], &s[1], &s[2]);
                double r2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
                if (r2 > t->ru2) continue;
                int ityj = ityp[j];
                int ktab = t->kpair[(ityj - 1) * ng + (ityi - 1)] - 1;
                int ktab1 = t->kpair[(ityi - 1) * ng + (ityj - 1)] - 1;
                double r = sqrt(r2);
                double sk = sqrt(r) * t->csi;
                int kk = (int)sk;
                double dk = sk - kk;
                double fortot = interp(t->fpotr, nk, nt, ktab, kk, dk) / r2 +
                                (interp(t->fpotb, nk, nt, ktab, kk, dk) * denki +
                                 interp(t->fpotb, nk, nt, ktab1, kk, dk) * den[j]) / r;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) p[3 * a + b] += s[a] * s[b] * fortot;
            }
        }
        for (int m = 0; m < 9; ++m) ap[(size_t)m * (size_t)n + (size_t)ic] = p[m];
    }
}

/* ------------------------------------------------------------------------------------ */
/* Hessian-vector product of the table-mode force                                        */
/* ------------------------------------------------------------------------------------ */
/* For a pair with separation s (|s| = R), SK = CSI sqrt(R), I_T = T(KK) + DK dT with
 * dT = T(KK+1) - T(KK), and dSK/dR = CSI / (2 sqrt(R)):
 *   rho_i = sum_j I_POTB,   rho_i' = sum_j dPOTB dSK/dR Rdot,   Rdot = s.(v_i - v_j) / R
 *   FS:  D = -1/(2 sqrt(rho)),  Ddot = rho^(-3/2) rhodot / 4
 *   EAM: D = I_DFEMBD(rho/RHOD + 1),  Ddot = dDFEMBD rhodot / RHOD
 *   F_i = sum_j FT s,  FT = I_FPOTR / R^2 + (I_FPOTB(k) D_i + I_FPOTB(k1) D_j) / R
 *   Fdot_i = sum_j FTdot s + FT (v_i - v_j),   hv = -Fdot.                              */
int orc_hvp(int n, const double *x, const double *y, const double *z, const int *ityp,
            const int *statu, const orc_box *box, const int *kvois, const int *indi, int ldi,
            const orc_tables *t, const double *vx, const double *vy, const double *vz,
            double *hx, double *hy, double *hz, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const double bx = box->len[0], by = box->len[1], bz = box->len[2];
    const double hbx = 0.5 * bx, hby = 0.5 * by, hbz = 0.5 * bz;
    const int px = box->ifpd[0], py = box->ifpd[1], pz = box->ifpd[2];
    const int nk = t->nkind, nt = t->ntab, ng = t->ngroup;
    size_t nn = (size_t)(n > 0 ? n : 1);
    double *dn = (double *)malloc(sizeof(double) * nn);
    double *dd = (double *)malloc(sizeof(double) * nn);
    int nbad = 0;

#pragma omp parallel for schedule(static) reduction(+ : nbad)
    for (int ic = 0; ic < n; ++ic) {
        double rho = 0.0, rhod = 0.0;
        int ityi = ityp[ic];
        dn[ic] = 0.0;
        dd[ic] = 0.0;
        if ((statu[ic] & ORC_STATU_ACTIVE) != ORC_STATU_ACTIVE) continue;
        for (int iw = 0; iw < kvois[ic]; ++iw) {
            int j = indi[(size_t)iw * (size_t)ldi + (size_t)ic];
            double sx = min_image(x[ic] - x[j], bx, hbx, px);
            double sy = min_image(y[ic] - y[j], by, hby, py);
            double sz = min_image(z[ic] - z[j], bz, hbz, pz);
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 > t->ru2) continue;
            int ktab = t->kpair[(ityp[j] - 1) * ng + (ityi - 1)] - 1;
            double r = sqrt(r2), sr = sqrt(r);
            double sk = sr * t->csi;
            int kk = (int)sk;
            double dk = sk - kk;
            double rdot = (sx * (vx[ic] - vx[j]) + sy * (vy[ic] - vy[j]) + sz * (vz[ic] - vz[j])) / r;
            rho += interp(t->potb, nk, nt, ktab, kk, dk);
            rhod += slope(t->potb, nk, nt, ktab, kk) * (t->csi / (2.0 * sr)) * rdot;
        }
        if (t->pottype == ORC_FS) {
            if (rho > 0.0) {
                dn[ic] = -0.5 / sqrt(rho);
                dd[ic] = 0.25 * rhod / (rho * sqrt(rho));
            }
        } else if (rho > 0.0) {
            int ke = t->kembd[ityi - 1] - 1, bad = 0;
            double sl = 0.0;
            dn[ic] = embd_lookup(t->dfembd, t->nkind1, t->nembd, ke, rho, t->rhod, &bad, &sl);
            dd[ic] = sl * rhod / t->rhod;
            nbad += bad;
        }
    }

#pragma omp parallel for schedule(static)
    for (int ic = 0; ic < n; ++ic) {
        double gx = 0.0, gy = 0.0, gz = 0.0;
        int ityi = ityp[ic];
        if ((statu[ic] & ORC_STATU_ACTIVE) == ORC_STATU_ACTIVE) {
            double di = dn[ic], ddi = dd[ic];
            for (int iw = 0; iw < kvois[ic]; ++iw) {
                int j = indi[(size_t)iw * (size_t)ldi + (size_t)ic];
                double sx = min_image(x[ic] - x[j], bx, hbx, px);
                double sy = min_image(y[ic] - y[j], by, hby, py);
                double sz = min_image(z[ic] - z[j], bz, hbz, pz);
                double r2 = sx * sx + sy * sy + sz * sz;
                if (r2 > t->ru2) continue;
                int ityj = ityp[j];
                int ktab = t->kpair[(ityj - 1) * ng + (ityi - 1)] - 1;
                int ktab1 = t->kpair[(ityi - 1) * ng + (ityj - 1)] - 1;
                double r = sqrt(r2), sr = sqrt(r);
                double sk = sr * t->csi;
                int kk = (int)sk;
                double dk = sk - kk;
                double skr = t->csi / (2.0 * sr);
                double wx = vx[ic] - vx[j], wy = vy[ic] - vy[j], wz = vz[ic] - vz[j];
                double rdot = (sx * wx + sy * wy + sz * wz) / r;
                double dj = dn[j], ddj = dd[j];
                double P = interp(t->fpotr, nk, nt, ktab, kk, dk);
                double B = interp(t->fpotb, nk, nt, ktab, kk, dk);
                double B1 = interp(t->fpotb, nk, nt, ktab1, kk, dk);
                double Pp = slope(t->fpotr, nk, nt, ktab, kk) * skr;
                double Bp = slope(t->fpotb, nk, nt, ktab, kk) * skr;
                double B1p = slope(t->fpotb, nk, nt, ktab1, kk) * skr;
                double emb = B * di + B1 * dj;
                double ft = P / r2 + emb / r;
                double dft_dr = Pp / r2 - 2.0 * P / (r2 * r) + (Bp * di + B1p * dj) / r - emb / r2;
                double ftdot = dft_dr * rdot + (B * ddi + B1 * ddj) / r;
                gx += ftdot * sx + ft * wx;
                gy += ftdot * sy + ft * wy;
                gz += ftdot * sz + ft * wz;
            }
        }
        hx[ic] = -gx;
        hy[ic] = -gy;
        hz[ic] = -gz;
    }
    free(dn);
    free(dd);
    return nbad;
}

/* ------------------------------------------------------------------------------------ */
/* force-matching gradient (forward mode, independent of the device adjoint)            */
/* ------------------------------------------------------------------------------------ */

/* complex-step derivative of the Cleri-Rosato table columns: with theta_m -> theta_m + i h,
 * Im(f)/h is the exact derivative to rounding. */
int orc_cr_dtables(const double *prm, double rmax, int ntab, double *d)
{
    const double csiv = 1.0 / ((double)ntab / sqrt(rmax));
    for (int m = 0; m < 5; ++m) {
        double h = 1e-30 * fabs(prm[m]);
        for (int i = 1; i <= ntab; ++i) {
            double t = (double)i * csiv;
            double r = t * t;
            double complex q[5];
            for (int k = 0; k < 5; ++k) q[k] = prm[k];
            q[m] += I * h;
            double complex A = q[0], xi = q[1], P = q[2], Q = q[3], r0 = q[4];
            double complex v = A * cexp(-P * ((r / r0) - 1.0));
            double complex fpotr = 2.0 * v * (P / r0) * r;
            double complex rho = (xi * xi) * cexp(-(2.0 * Q) * ((r / r0) - 1.0));
            double complex fpotb = rho * (Q / r0) * 2.0;
            d[(size_t)(m * 3 + 0) * ntab + (i - 1)] = cimag(fpotr) / h;
            d[(size_t)(m * 3 + 1) * ntab + (i - 1)] = cimag(rho) / h;
            d[(size_t)(m * 3 + 2) * ntab + (i - 1)] = cimag(fpotb) / h;
        }
    }
    return 0;
}

int orc_adjoint_cr(int n, const double *x, const double *y, const double *z, const int *ityp,
                   const int *statu, const orc_box *box, const int *kvois, const int *indi,
                   int ldi, const orc_tables *t, const double *dtab, const double *ftx,
                   const double *fty, const double *ftz, double *loss, double *grad,
                   int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    size_t nn = (size_t)(n > 0 ? n : 1);
    double *fx = (double *)malloc(sizeof(double) * nn), *fy = (double *)malloc(sizeof(double) * nn);
    double *fz = (double *)malloc(sizeof(double) * nn), *dn = (double *)malloc(sizeof(double) * nn);
    double *rho = (double *)calloc(nn, sizeof(double)), *drho = (double *)calloc(nn, sizeof(double));
    orc_force(n, x, y, z, ityp, statu, box, kvois, indi, ldi, t, dn, fx, fy, fz, NULL, NULL, nthreads);
    double l = 0.0;
    for (int i = 0; i < n; ++i) {
        double a = fx[i] - ftx[i], b = fy[i] - fty[i], c = fz[i] - ftz[i];
        l += a * a + b * b + c * c;
    }
    *loss = l;
    const double bx = box->len[0], by = box->len[1], bz = box->len[2];
    const int px = box->ifpd[0], py = box->ifpd[1], pz = box->ifpd[2];
    const int nt = t->ntab;
    for (int m = 0; m < 5; ++m) {
        const double *dP = dtab + (size_t)(m * 3 + 0) * nt;
        const double *dQ = dtab + (size_t)(m * 3 + 1) * nt;
        const double *dB = dtab + (size_t)(m * 3 + 2) * nt;
        /* d rho_i / d theta_m and d F'_i / d theta_m */
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            double r0 = 0.0, d0 = 0.0;
            if ((statu[i] & ORC_STATU_ACTIVE) == ORC_STATU_ACTIVE) {
                for (int w = 0; w < kvois[i]; ++w) {
                    int j = indi[(size_t)w * (size_t)ldi + (size_t)i];
                    double sx = min_image(x[i] - x[j], bx, 0.5 * bx, px);
                    double sy = min_image(y[i] - y[j], by, 0.5 * by, py);
                    double sz = min_image(z[i] - z[j], bz, 0.5 * bz, pz);
                    double r2 = sx * sx + sy * sy + sz * sz;
                    if (r2 > t->ru2) continue;
                    double sk = sqrt(sqrt(r2)) * t->csi;
                    int kk = (int)sk;
                    double dk = sk - kk;
                    r0 += interp(t->potb, 1, nt, 0, kk, dk);
                    d0 += interp(dQ, 1, nt, 0, kk, dk);
                }
            }
            rho[i] = r0;
            drho[i] = r0 > 0.0 ? 0.25 * d0 / (r0 * sqrt(r0)) : 0.0;   /* dD_i */
        }
        double g = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : g)
        for (int i = 0; i < n; ++i) {
            if ((statu[i] & ORC_STATU_ACTIVE) != ORC_STATU_ACTIVE) continue;
            double gx = 0.0, gy = 0.0, gz = 0.0;
            for (int w = 0; w < kvois[i]; ++w) {
                int j = indi[(size_t)w * (size_t)ldi + (size_t)i];
                double sx = min_image(x[i] - x[j], bx, 0.5 * bx, px);
                double sy = min_image(y[i] - y[j], by, 0.5 * by, py);
                double sz = min_image(z[i] - z[j], bz, 0.5 * bz, pz);
                double r2 = sx * sx + sy * sy + sz * sz;
                if (r2 > t->ru2) continue;
                double r = sqrt(r2);
                double sk = sqrt(r) * t->csi;
                int kk = (int)sk;
                double dk = sk - kk;
                double B = interp(t->fpotb, 1, nt, 0, kk, dk);
                double dft = interp(dP, 1, nt, 0, kk, dk) / r2 +
                             (interp(dB, 1, nt, 0, kk, dk) * (dn[i] + dn[j]) +
                              B * (drho[i] + drho[j])) / r;
                gx += dft * sx;
                gy += dft * sy;
                gz += dft * sz;
            }
            g += (fx[i] - ftx[i]) * gx + (fy[i] - fty[i]) * gy + (fz[i] - ftz[i]) * gz;
        }
        grad[m] = 2.0 * g;
    }
    free(fx); free(fy); free(fz); free(dn); free(rho); free(drho);
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Natural cubic spline (the interpolant of SLATEC DBINT4 with IBCL = IBCR = 2, FBCL =    */
/* FBCR = 0, KNTOPT = 1, used by Filedatas_Func_Setfl.F90:256-276), uniform grid           */
/* ------------------------------------------------------------------------------------ */
void orc_spline_natural(int n, double h, const double *y, double *m)
{
    /* m_{i-1} + 4 m_i + m_{i+1} = 6 (y_{i+1} - 2 y_i + y_{i-1}) / h^2, m_0 = m_{n-1} = 0,
     * solved by forward elimination / back substitution (Thomas) */
    if (n < 3) {
        for (int i = 0; i < n; ++i) m[i] = 0.0;
        return;
    }
    double *cp = (double *)malloc(sizeof(double) * (size_t)n);
    const double s = 6.0 / (h * h);
    m[0] = 0.0;
    cp[0] = 0.0;
    for (int i = 1; i < n - 1; ++i) {
        const double rhs = s * (y[i + 1] - 2.0 * y[i] + y[i - 1]);
        const double den = 4.0 - cp[i - 1];
        cp[i] = 1.0 / den;
        m[i] = (rhs - m[i - 1]) / den;
    }
    m[n - 1] = 0.0;
    for (int i = n - 2; i >= 1; --i) m[i] -= cp[i] * m[i + 1];
    free(cp);
}

double orc_spline_eval(int n, double x0, double h, const double *y, const double *m, double x,
                       double *dy)
{
    int k = (int)floor((x - x0) / h);
    if (k < 0) k = 0;
    if (k > n - 2) k = n - 2;
    const double xk = x0 + k * h;
    const double b = (x - xk) / h, a = 1.0 - b;
    const double h26 = h * h / 6.0;
    if (dy)
        *dy = (y[k + 1] - y[k]) / h + h * ((1.0 - 3.0 * a * a) * m[k] + (3.0 * b * b - 1.0) * m[k + 1]) / 6.0;
    return a * y[k] + b * y[k + 1] + ((a * a * a - a) * m[k] + (b * b * b - b) * m[k + 1]) * h26;
}

void orc_spline_knots(int n, const double *x, const double *y, double *m)
{
    /* mu_i m_{i-1} + 2 m_i + lam_i m_{i+1} = d_i with mu_i = h_{i-1}/(h_{i-1}+h_i),
     * lam_i = 1 - mu_i, d_i = 6 [x_{i-1}, x_i, x_{i+1}] (second divided difference) */
    double *c = (double *)calloc((size_t)n, sizeof(double));
    for (int i = 0; i < n; ++i) m[i] = 0.0;
    for (int i = 1; i < n - 1; ++i) {
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        const double mu = h0 / (h0 + h1), lam = 1.0 - mu;
        const double d = 6.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0) / (h0 + h1);
        const double piv = 2.0 - mu * c[i - 1];
        c[i] = lam / piv;
        m[i] = (d - mu * m[i - 1]) / piv;
    }
    for (int i = n - 2; i > 0; --i) m[i] -= c[i] * m[i + 1];
    free(c);
}

void orc_spline_knots_eval(int n, const double *x, const double *y, const double *m, int nt,
                           const double *t, double *f, double *df)
{
    for (int k = 0; k < nt; ++k) {
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (t[k] >= x[mid]) lo = mid; else hi = mid;
        }
        const double h = x[hi] - x[lo];
        const double u = x[hi] - t[k], v = t[k] - x[lo];
        f[k] = (m[lo] * u * u * u + m[hi] * v * v * v) / (6.0 * h) + (y[lo] / h - m[lo] * h / 6.0) * u +
               (y[hi] / h - m[hi] * h / 6.0) * v;
        df[k] = (m[hi] * v * v - m[lo] * u * u) / (2.0 * h) + (y[hi] - y[lo]) / h - (m[hi] - m[lo]) * h / 6.0;
    }
}

int orc_setfl_tables(int nrho, double drho, int nr, double cutoff, const double *frho,
                     const double *rhor, const double *rphi, int ntab, double *potr, double *fpotr,
                     double *potb, double *fpotb, double *fembd, double *dfembd)
{
    if (nrho < 3 || nr < 3 || ntab < 2) return -1;
    const double dr = cutoff / nr;              /* R(I) = (I-1) cutoff/Nr (:166-169) */
    const double rimax = (nr - 1) * dr, fimax = (nrho - 1) * drho;
    double *m1 = (double *)malloc(sizeof(double) * (size_t)nr);
    double *m2 = (double *)malloc(sizeof(double) * (size_t)nr);
    double *m3 = (double *)malloc(sizeof(double) * (size_t)nrho);
    orc_spline_natural(nr, dr, rphi, m1);
    orc_spline_natural(nr, dr, rhor, m2);
    orc_spline_natural(nrho, drho, frho, m3);
    int fzero = 1;
    for (int i = 0; i < nrho; ++i)
        if (frho[i] != 0.0) fzero = 0;
    const double csiv = sqrt(cutoff) / ntab;
    for (int i = 1; i <= ntab; ++i) {
        const double t = i * csiv, r = t * t;
        double f = 0.0, df = 0.0, rho = 0.0, drh = 0.0;
        if (r <= rimax) {                       /* Vr_Spline / Rhor_Spline; zero beyond */
            f = orc_spline_eval(nr, 0.0, dr, rphi, m1, r, &df);
            if (!fzero) rho = orc_spline_eval(nr, 0.0, dr, rhor, m2, r, &drh);
        }
        const double phi = f / r;               /* NN_Spline: V = (r phi)/r, V' = (F' - V)/r */
        const double dphi = (df - phi) / r;
        potr[i - 1] = 0.5 * phi * r;
        fpotr[i - 1] = -dphi * r;
        potb[i - 1] = rho;
        fpotb[i - 1] = -drh;
    }
    for (int i = 1; i <= nrho; ++i) {           /* EMBED_Spline on RHO_i = (i-1) RHOD, RHOD = drho */
        const double rho = (i - 1) * drho;
        double d = 0.0, f;
        if (rho <= fimax) {
            f = orc_spline_eval(nrho, 0.0, drho, frho, m3, rho, &d);
        } else {
            f = orc_spline_eval(nrho, 0.0, drho, frho, m3, fimax, NULL);
            d = 0.0;
        }
        fembd[i - 1] = f;
        dfembd[i - 1] = d;
    }
    free(m1);
    free(m2);
    free(m3);
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Re-grid of imported tables (Register_Imported_ForceTable, MD_TypeDef_ForceTable.F90:    */
/* 1612-1855) through SPLID1 / SPLID2 (LIB/sor/f/MiniUtilities/DINTF2.F:17-240) with       */
/* IOP(1) = IOP(2) = 5 and IJ = 1                                                          */
/* ------------------------------------------------------------------------------------ */

/* SPLID1 with IOP = 5 at both ends: the end first derivatives are those of the cubic through
 * the four end points (DINTF2.F:75-96), and option 5 then proceeds as the clamped option 3
 * (:120-130, 170-178).  The second derivatives w solve
 *   row 1:      2 h_1 w_1 + h_1 w_2                       = 6 (D_1 - C1)
 *   row i:      h_{i-1} w_{i-1} + 2 (h_{i-1} + h_i) w_i + h_i w_{i+1} = 6 (D_i - D_{i-1})
 *   row N:      h_{N-1} w_{N-1} + 2 h_{N-1} w_N            = 6 (C2 - D_{N-1})
 * with h_i = x_{i+1} - x_i, D_i = (f_{i+1} - f_i)/h_i; solved here by forward elimination
 * and back substitution.  Requires n >= 4 (the reference prints a warning otherwise). */
void orc_splid1(int n, const double *x, const double *f, double *w)
{
    const double a1 = x[0] - x[1], a2 = x[0] - x[2], a3 = x[0] - x[3];
    const double a4 = x[1] - x[2], a5 = x[1] - x[3], a6 = x[2] - x[3];
    const double c1 = f[0] * (1.0 / a1 + 1.0 / a2 + 1.0 / a3) - a2 * a3 * f[1] / (a1 * a4 * a5) +
                      a1 * a3 * f[2] / (a2 * a4 * a6) - a1 * a2 * f[3] / (a3 * a5 * a6);
    const double b1 = x[n - 1] - x[n - 4], b2 = x[n - 1] - x[n - 3], b3 = x[n - 1] - x[n - 2];
    const double b4 = x[n - 2] - x[n - 4], b5 = x[n - 2] - x[n - 3], b6 = x[n - 3] - x[n - 4];
    const double c2 = -b2 * b3 * f[n - 4] / (b6 * b4 * b1) + b1 * b3 * f[n - 3] / (b6 * b5 * b2) -
                      b1 * b2 * f[n - 2] / (b4 * b5 * b3) + f[n - 1] * (1.0 / b1 + 1.0 / b2 + 1.0 / b3);
    double *cp = (double *)malloc(sizeof(double) * (size_t)n);
    double *rp = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        double lo = 0.0, di, up = 0.0, r;
        if (i == 0) {
            const double h = x[1] - x[0];
            di = 2.0 * h;
            up = h;
            r = 6.0 * ((f[1] - f[0]) / h - c1);
        } else if (i == n - 1) {
            const double h = x[n - 1] - x[n - 2];
            lo = h;
            di = 2.0 * h;
            r = 6.0 * (c2 - (f[n - 1] - f[n - 2]) / h);
        } else {
            const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
            lo = h0;
            di = 2.0 * (h0 + h1);
            up = h1;
            r = 6.0 * ((f[i + 1] - f[i]) / h1 - (f[i] - f[i - 1]) / h0);
        }
        const double piv = i > 0 ? di - lo * cp[i - 1] : di;
        cp[i] = up / piv;
        rp[i] = (i > 0 ? r - lo * rp[i - 1] : r) / piv;
    }
    w[n - 1] = rp[n - 1];
    for (int i = n - 2; i >= 0; --i) w[i] = rp[i] - cp[i] * w[i + 1];
    free(cp);
    free(rp);
}

/* SPLID2 (DINTF2.F:176-218): the interval I with X(I) <= Y < X(I+1) (SEARCH), I = 1 for
 * Y <= X(1) and I = N-1 for Y >= X(N), then the cubic of that interval at Y. */
double orc_splid2(int n, const double *x, const double *f, const double *w, double y)
{
    int i;
    if (y <= x[0]) {
        i = 0;
    } else if (y >= x[n - 1]) {
        i = n - 2;
    } else {
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (y >= x[mid]) lo = mid; else hi = mid;
        }
        i = lo;
    }
    const double flk = x[i + 1] - x[i];
    const double u = x[i + 1] - y, v = y - x[i];
    const double a = (w[i] * u * u * u + w[i + 1] * v * v * v) / (6.0 * flk);
    const double b = (f[i + 1] / flk - w[i + 1] * flk / 6.0) * v;
    const double c = (f[i] / flk - flk * w[i] / 6.0) * u;
    return a + b + c;
}

/* one pair column on the run's grid (:1714-1724 and its three twins): T = K CSIV with
 * CSIV = 1/CSI, CSI = NTAB/sqrt(Rmax) (New_ForceTable :591-594); 0 where T^2 > max R */
void orc_import_regrid_pair(int nf, const double *rf, const double *yf, double rmax, int ntab, double *out)
{
    double *w = (double *)malloc(sizeof(double) * (size_t)nf);
    orc_splid1(nf, rf, yf, w);
    double trmax = rf[0];
    for (int i = 1; i < nf; ++i)
        if (rf[i] > trmax) trmax = rf[i];
    const double csi = (double)ntab / sqrt(rmax), csiv = 1.0 / csi;
    for (int k = 1; k <= ntab; ++k) {
        const double t = (double)k * csiv, tt = t * t;
        out[k - 1] = tt <= trmax ? orc_splid2(nf, rf, yf, w, tt) : 0.0;
    }
    free(w);
}

/* one embedding column (:1818-1830): rho = (K-1) RHOD, no range test */
void orc_import_regrid_embd(int nf, const double *rhof, const double *yf, double rhod, int nembd, double *out)
{
    double *w = (double *)malloc(sizeof(double) * (size_t)nf);
    orc_splid1(nf, rhof, yf, w);
    for (int k = 1; k <= nembd; ++k) out[k - 1] = orc_splid2(nf, rhof, yf, w, (double)(k - 1) * rhod);
    free(w);
}
