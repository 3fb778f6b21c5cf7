/*
 * msm_oracle.h -- CPU restatement of the msmpscu many-body force / neighbour-list /
 * velocity-Verlet path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * CPU-baseline leg of bench.py call it as the checker.  The product library never links it.
 *
 * Parity status: the table generator is pinned against the reference's exported force-table
 * fixture (examples/use_ForceTableGen/EM_TB_WANGJUN_W-HE_2010.pair, W-W Ackland-Thetford
 * columns).  Forces, energies, virial, neighbour sets and the integrator have no reference
 * golden vectors (the reference ships none, and its Fortran cannot be compiled here), so
 * their parity is "unpinned" beyond the restatement itself plus physical invariants
 * (sum F = 0, energy/force finite differences, lattice symmetry).
 *
 * Units are whatever the caller uses consistently (the tests use Angstrom, eV, fs and
 * masses in eV*fs^2/A^2); the reference itself runs in CGS.
 *
 * Table layout follows the reference's MDForceTable (MD_TypeDef_ForceTable.F90:117-155):
 * column-major (NKIND, NTAB), i.e. entry (kind k, point i) [both 1-based] lives at
 * T[(i-1)*nkind + (k-1)].  Grid point i sits at r_i = (i/CSI)^2.
 */
#ifndef MSM_ORACLE_H
#define MSM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* status bits, MD_Const.F90:78-96 */
#define ORC_STATU_ACTIVE    1
#define ORC_STATU_FIXPOSX   2
#define ORC_STATU_FIXPOSY   4
#define ORC_STATU_FIXPOSZ   8
#define ORC_STATU_FIXVELX   16
#define ORC_STATU_FIXVELY   32
#define ORC_STATU_FIXVELZ   64
#define ORC_STATU_OUTOFBOX  65536
#define ORC_STATU_REFLECT   131072
#define ORC_STATU_TRANSMIT  262144
#define ORC_STATU_PASSBOUND 524288

/* potential ids understood by orc_pot_eval / orc_make_tables */
#define ORC_POT_CR          1   /* Cleri-Rosato TB-SMA (FS form); prm = A, xi, p, q, r0 */
#define ORC_POT_MARINICA2   2   /* Marinica EAM2 W (EAM form); prm unused */
#define ORC_POT_ACKLAND_WW  3   /* Ackland-Thetford W (FS form); prm unused; Angstrom/eV units */
#define ORC_POT_DERLET_WW   4   /* Derlet-Nguyen-Manh-Dudarev W (FS form), FS_PM_WW.F90 */
#define ORC_POT_HEHE_EXP6   5   /* He-He ZBL / cubic / EXP6 (no density), ZBL_EXP6_HeHe.F90 */
#define ORC_POT_HEW_ZBL     6   /* He-W ZBL / cubics / EXP6 (no density), ZBL_ABINTIO_He_W_930.F90 */
#define ORC_POT_MARINICA3   7   /* Marinica EAM3 W (EAM form), EAM3_WW_Marinica_JPCM25_2013.F90 */
#define ORC_POT_MARINICA4   8   /* Marinica EAM4 W (EAM form), EAM4_WW_Marinica_JPCM25_2013.F90 */
#define ORC_POT_AV_CU       9   /* Ackland-Vitek Cu (FS form), EM_TB_CuCu_Ackland_Vitek_PRB41_10324.F90 */
#define ORC_POT_AV_AU      10   /* Ackland-Vitek Au (FS form), EM_TB_AuAu_Ackland_Vitek_PRB41_10324.F90 */
#define ORC_POT_AV_CUAU    11   /* Ackland-Vitek Cu-Au (FS form), EM_TB_CuAu_Ackland_Vitek_PRB41_10324.F90 */
#define ORC_POT_MENDELEV_ZR 12  /* Mendelev-Ackland Zr (EAM form), EAM_ZrZr_Mendelev_Phil_Mag_L87_2007.F90 */
#define ORC_POT_AWB_ZR     13   /* Ackland-Wooding-Bacon Zr (FS form), EM_TB_AWB_Phil_Mag_A71_1995_553.F90 */
#define ORC_POT_HETI_LJ    14   /* He-Ti pair (no density), EM_TB_WangJun_Ti-HE_2007/LJ_He_Ti.F90 */

#define ORC_FS  0
#define ORC_EAM 1

typedef struct {
    int pottype;          /* ORC_FS or ORC_EAM */
    int ntab, nkind;
    double csi;           /* NTAB / sqrt(Rmax) */
    double ru2;           /* max cutoff squared */
    const double *potr, *fpotr, *potb, *fpotb;   /* (nkind, ntab) column-major */
    int nembd, nkind1;
    double rhod;
    const double *fembd, *dfembd;                /* (nkind1, nembd) column-major */
    int ngroup;
    const int *kpair;     /* (ngroup, ngroup) column-major, 1-based table ids  */
    const int *kembd;     /* (ngroup), 1-based embedding table ids             */
} orc_tables;

typedef struct {
    double lo[3];
    double len[3];
    int ifpd[3];
    int shaped;           /* nonzero: separations are BOXSHAPE . SEP (MD_FS_ForceTable.F90:235,333) */
    double bs[9];         /* BOXSHAPE(K, 1:3) in row K */
} orc_box;

/* potential functions: value and -derivative in the reference's conventions */
int  orc_pot_eval(int pot, const double *prm, double r, double *potr, double *fpotr,
                  double *potb, double *fpotb);
int  orc_embed_eval(int pot, const double *prm, double rho, double *f, double *df);

/* table generator (MD_TypeDef_ForceTable.F90:530-622, 890-1056); single species.
 * potr..fpotb have ntab entries, fembd/dfembd nembd entries (may be NULL for FS).
 * Returns RHOD through *rhod (RHOMX = rhoscal * max POTB). */
int  orc_make_tables(int pot, const double *prm, double rmax, int ntab, int nembd, double rhoscal,
                     double *potr, double *fpotr, double *potb, double *fpotb,
                     double *fembd, double *dfembd, double *rhod);

/* Tabulated EAM potentials in LAMMPS setfl layout (Filedatas_Func_Setfl.F90:119-253).  The
 * reference interpolates the file's arrays with SLATEC DBINT4/DBVALU (LIB/sor/f/MATH90A) with
 * IBCL = IBCR = 2, FBCL = FBCR = 0, KNTOPT = 1 (:25-34): the cubic interpolating spline with
 * knots at the data points and zero second derivative at both ends, i.e. the natural cubic
 * spline, restated here on the uniform grid x_i = x0 + i h.
 *   orc_spline_natural: second derivatives m[0..n-1] (m[0] = m[n-1] = 0)
 *   orc_spline_eval:    value (and derivative through *dy) at x in [x0, x0 + (n-1) h]   */
void   orc_spline_natural(int n, double h, const double *y, double *m);
double orc_spline_eval(int n, double x0, double h, const double *y, const double *m, double x,
                       double *dy);
/* One element's pair and embedding tables from setfl arrays (r grid R_i = i cutoff/nr,
 * rho grid (i) drho, rphi = r*phi(r)), on the sqrt(r) grid of ntab points up to
 * Rmax = cutoff and the rho grid RHOD = drho of nrho points (the file's own grid):
 *   POTR = 0.5 r phi, FPOTR = -r dphi/dr (NN_Spline, :440-458), POTB = rho(r),
 *   FPOTB = -drho/dr (RHO_Spline, :461-476), FEMBD/DFEMBD = F, dF/drho (EMBED_Spline,
 *   :479-496), with the reference's clamping outside the data range (:292-437). */
int    orc_setfl_tables(int nrho, double drho, int nr, double cutoff, const double *frho,
                        const double *rhor, const double *rphi, int ntab, double *potr, double *fpotr,
                        double *potb, double *fpotb, double *fembd, double *dfembd);

/* Bonny W-H-He EAM (EAM1_WHeH_Bonny_JPCM26_2014.F90, EAM_ForceTable_Bonny_JPCM26_2014.F90):
 * pair/density functions of table t (registration order, 1-based) and the embedding of group g
 * (1 W, 2 H, 3 He) for subtype sub (1 EAM1, 2 EAM2), Angstrom / eV, POTR = V/2 conventions. */
int    orc_bonny_pair(int sub, int t, double r, double *potr, double *fpotr, double *potb, double *fpotb);
int    orc_bonny_embed(int sub, int g, double rho, double *f, double *df);

/* The same natural cubic spline on arbitrary increasing knots x_0 < ... < x_{n-1} (the lspt
 * ".spt" files, Filedatas_Func_Lspt.F90:304-324 with the settings of :24-34):
 *   orc_spline_knots:      second derivatives m (m[0] = m[n-1] = 0)
 *   orc_spline_knots_eval: value f[k] and derivative df[k] at each t[k] in [x_0, x_{n-1}] */
void   orc_spline_knots(int n, const double *x, const double *y, double *m);
void   orc_spline_knots_eval(int n, const double *x, const double *y, const double *m, int nt,
                             const double *t, double *f, double *df);

/* neighbour list (MD_NeighborsList.F90:396-633/* neighbour list (MD_NeighborsList.F90:396-633, cut rule d^2 < rc^2 in FP64, minimum image).
 * indi is ELL column-major: neighbour k of atom i at indi[k*n + i]; 0-based atom ids.
 * Returns 0, or -1 on neighbour overflow, -2 on an atom outside the box. */
int  orc_nlist(int n, const double *x, const double *y, const double *z, const int *statu,
               const orc_box *box, double rc_nl, int mxkvois, int *kvois, int *indi, int *ncell3);

/* brute-force O(N^2) minimum-image neighbour sets (same cut rule), for cross-checks */
int  orc_nlist_brute(int n, const double *x, const double *y, const double *z, const int *statu,
                     const orc_box *box, double rc_nl, int mxkvois, int *kvois, int *indi);

/* force passes (MD_FS_ForceTable_GPU.F90:341-516, 623-806, 998-1272, 1451-1609 and the
 * EAM twins in MD_EAM_ForceTable_GPU.F90:369-548, 646-829, 1014-1289, 1470-1636).
 * den/fx/fy/fz/epot/vir9 may be NULL when not wanted.  Returns the number of atoms whose
 * embedding lookup fell outside the F(rho) table (EAM), else 0. */
int  orc_force(int n, const double *x, const double *y, const double *z, const int *ityp,
               const int *statu, const orc_box *box, const int *kvois, const int *indi, int ldi,
               const orc_tables *t, double *den, double *fx, double *fy, double *fz,
               double *epot, double *vir9, int nthreads);

/* per-atom virial tensor, CAL_FS_AtomicStress_KERNEL (MD_FS_ForceTable_GPU.F90:1746-1965) and
 * CAL_EAM_AtomicStress_KERNEL (MD_EAM_ForceTable_GPU.F90:1775-1994), cubic box:
 * AP(i, 3a+b) = sum_j FORTOT s_a s_b (no 1/2), zero on inactive atoms.  den = F'(rho) from
 * orc_force; ap has 9 slabs of n (the reference's AP(NAPDEV, 9) column-major). */
void orc_atomic_stress(int n, const double *x, const double *y, const double *z, const int *ityp,
                       const int *statu, const orc_box *box, const int *kvois, const int *indi,
                       int ldi, const orc_tables *t, const double *den, double *ap, int nthreads);

/* Swope velocity Verlet (MD_DiffScheme_GPU.F90:242-384 predictor, 686-760 corrector) */
void orc_predictor(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                   const double *fx, const double *fy, const double *fz, double *dx, double *dy,
                   double *dz, int *statu, const int *ityp, const double *cm, double h,
                   const orc_box *box);
void orc_corrector(int n, double *vx, double *vy, double *vz, const double *fx, const double *fy,
                   const double *fz, const int *statu, const int *ityp, const double *cm, double h);

/* NVE loop: list build, force, then nsteps of predictor / skin check / force / corrector.
 * The list is rebuilt when the largest displacement since the last build exceeds
 * skin_trigger (<= 0: rebuild every nb_uptab steps as the reference does).  Returns the
 * number of rebuilds after the initial one, or < 0 on error. */
int  orc_md(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
            double *fx, double *fy, double *fz, int *statu, const int *ityp, const orc_box *box,
            const orc_tables *t, const double *cm, double h, int nsteps, double rc_nl,
            double skin_trigger, int nb_uptab, int mxkvois, int nthreads);
/* orc_md with an external force fext (3n: x block, y block, z block; NULL for none) added to
 * every active atom after each force evaluation (Cumulate_ExtForce0) */
int  orc_md_ext(int n, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                double *fx, double *fy, double *fz, int *statu, const int *ityp, const orc_box *box,
                const orc_tables *t, const double *cm, double h, int nsteps, double rc_nl,
                double skin_trigger, int nb_uptab, int mxkvois, int nthreads, const double *fext);

/* Hessian-vector product of the table-mode force: hv = -dF/dx . v, with the exact
 * derivative of the piecewise-linear interpolants. */
int  orc_hvp(int n, const double *x, const double *y, const double *z, const int *ityp,
             const int *statu, const orc_box *box, const int *kvois, const int *indi, int ldi,
             const orc_tables *t, const double *vx, const double *vy, const double *vz,
             double *hx, double *hy, double *hz, int nthreads);

/* Cleri-Rosato parameter derivatives of FPOTR, POTB, FPOTB on the table grid, by complex-step
 * differentiation of the potential functions: d[(m*3 + t)*ntab + i-1]. */
int  orc_cr_dtables(const double *prm, double rmax, int ntab, double *d);

/* Force-matching gradient by forward mode: for each parameter, dF/dtheta of every atom
 * through the tables and the FS embedding, dotted with w = F - Ft (active atoms).
 * dtab from orc_cr_dtables.  Returns L = sum |F - Ft|^2 and grad[5] = dL/dtheta. */
int  orc_adjoint_cr(int n, const double *x, const double *y, const double *z, const int *ityp,
                    const int *statu, const orc_box *box, const int *kvois, const int *indi,
                    int ldi, const orc_tables *t, const double *dtab, const double *ftx,
                    const double *fty, const double *ftz, double *loss, double *grad,
                    int nthreads);

/* Re-grid of imported tables (Register_Imported_ForceTable, MD_TypeDef_ForceTable.F90:1612-1855)
 * through SPLID1/SPLID2 (LIB/sor/f/MiniUtilities/DINTF2.F) with end slopes from the four end
 * points (IOP = 5):
 *   orc_splid1: second derivatives w of the spline through (x, f), n >= 4
 *   orc_splid2: its value at y (end intervals extended)
 *   orc_import_regrid_pair: a pair column onto T = K/CSI, K = 1..ntab (0 beyond max r)
 *   orc_import_regrid_embd: an embedding column onto rho = (K-1) rhod, K = 1..nembd        */
void   orc_splid1(int n, const double *x, const double *f, double *w);
double orc_splid2(int n, const double *x, const double *f, const double *w, double y);
void   orc_import_regrid_pair(int nf, const double *rf, const double *yf, double rmax, int ntab, double *out);
void   orc_import_regrid_embd(int nf, const double *rhof, const double *yf, double rhod, int nembd, double *out);

#ifdef __cplusplus
}
#endif
#endif
