/*
 * msmgb.h -- C ABI of the GB300 many-body MD hot path (libmsmgb.so).
 *
 * The entry points replace the CUDA Fortran routines that msmpscu's MD loop calls through
 * its force class (MDForceClassGPU, MD_ForceClass_Register_GPU.F90:248-259), its GPU
 * neighbour list (MD_NeighborsList_GPU.F90) and its GPU integrator (MD_DiffScheme_GPU.F90).
 * All arguments are plain C types; host arrays are read or written only during the call.
 * Every function returns MSMGB_OK (0) or a negative MSMGB_ERR_* code; the message of the
 * last failure is available through msmgb_last_error().
 *
 * Units: the library is unit-agnostic.  Positions, box, cutoffs, tables, masses and time
 * step must be given in one consistent system (msmpscu's host uses CGS; the tests use
 * Angstrom, eV, fs and masses in eV*fs^2/A^2).  Per-atom arrays use the reference's layout:
 * XP(N,3) column-major, i.e. x[0..N), y[N..2N), z[2N..3N); atom types ITYP are 1-based.
 *
 * Threading: one context per host thread; a context is not thread-safe.  All device work
 * of a context is issued on one CUDA stream (msmgb_stream()).
 */
#ifndef MSMGB_H
#define MSMGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace the reference's `stop` statements) ------------------------ */
#define MSMGB_OK                 0
#define MSMGB_ERR_ARG           -1   /* bad argument / call order                          */
#define MSMGB_ERR_CUDA          -2   /* CUDA runtime error (message has the CUDA text)     */
#define MSMGB_ERR_NL_OVERFLOW   -3   /* an atom has more than MXKVOIS neighbours           */
#define MSMGB_ERR_OUT_OF_BOX    -4   /* an active atom lies outside its box (cell binning) */
#define MSMGB_ERR_RHO_RANGE     -5   /* EAM: density beyond the F(rho) table               */
#define MSMGB_ERR_BOX_TOO_SMALL -6   /* box edge < 2 * list cutoff (minimum image ambiguous)*/
#define MSMGB_ERR_NO_DEVICE     -7   /* no CUDA device / extension unusable                */
#define MSMGB_ERR_CAPACITY      -8   /* more atoms / boxes than the context was sized for  */
#define MSMGB_ERR_TIMEOUT       -9   /* a bounded device-side wait ran out (asynchronous copy
                                        not completed); the context stays usable            */

/* ---- potential types (MDForceTable%PotType) ------------------------------------------- */
#define MSMGB_FS_TYPE  0
#define MSMGB_EAM_TYPE 1

/* ---- arithmetic of the force passes ---------------------------------------------------- */
#define MSMGB_PREC_FP64  0   /* plain FP64, the reference's arithmetic                   */
#define MSMGB_PREC_MIXED 1   /* FP32 pair, density and table terms and sums on an exact
                                float-float table index (force error <= 1e-6 relative);
                                FP64 positions and integration                           */
#define MSMGB_PREC_FF    2   /* float-float (two FP32 numbers per value) force passes:
                                FP64 parity (<= 1e-10 relative) on the FP32 pipe; the
                                virial and per-atom energy calls use the FP64 passes     */

/* ---- atom status bits (MD_Const.F90:78-96) ---------------------------------------------- */
#define MSMGB_STATU_ACTIVE    1
#define MSMGB_STATU_FIXPOSX   2
#define MSMGB_STATU_FIXPOSY   4
#define MSMGB_STATU_FIXPOSZ   8
#define MSMGB_STATU_FIXVELX   16
#define MSMGB_STATU_FIXVELY   32
#define MSMGB_STATU_FIXVELZ   64
#define MSMGB_STATU_OUTOFBOX  65536
#define MSMGB_STATU_REFLECT   131072
#define MSMGB_STATU_TRANSMIT  262144

/* ---- output ordering -------------------------------------------------------------------- */
#define MSMGB_ORDER_ORIGINAL 0   /* the caller's atom order (reference: hm_GIDINV copy-out) */
#define MSMGB_ORDER_SORTED   1   /* the library's cell-sorted device order                 */

typedef struct msmgb_ctx msmgb_ctx;

/* Context parameters: the control-file fields of the neighbour list and integrator
 * (SimMDCtrl NB_RM, NB_MXNBS, NB_UPTAB; MD_TypeDef_SimCtrlParam.F90:116-123). */
typedef struct {
    int    device;        /* CUDA device ordinal                                          */
    int    max_atoms;     /* capacity: total atoms over all boxes                         */
    int    max_boxes;     /* capacity: number of boxes (1 for a single box)               */
    int    mxkvois;       /* NB_MXNBS: neighbour slots per atom (ELL width)               */
    double rc_nl;         /* NB_RM: neighbour-list cutoff (absolute length)               */
    double skin_trigger;  /* rebuild when max displacement since the last build exceeds
                             this (> 0); <= 0 selects the reference's fixed interval      */
    int    nb_uptab;      /* NB_UPTAB: rebuild interval when skin_trigger <= 0            */
    int    precision;     /* MSMGB_PREC_FP64, MSMGB_PREC_MIXED or MSMGB_PREC_FF           */
    void  *stream;        /* cudaStream_t to issue on; NULL = the context makes its own   */
} msmgb_params;

/* Force table: the MDForceTable fields the GPU passes read
 * (MD_TypeDef_ForceTable.F90:117-155).  Arrays are in the reference's column-major layout:
 * POTR(NKIND,NTAB) has entry (k,i) at potr[(i-1)*nkind + (k-1)].  Grid point i is at
 * r = (i*sqrt(rmax)/ntab)^2.  The EAM fields are ignored for MSMGB_FS_TYPE. */
typedef struct {
    int           pottype;          /* MSMGB_FS_TYPE or MSMGB_EAM_TYPE                     */
    int           ntab, nkind;
    double        rmax;             /* Rmax = max RU                                        */
    const double *potr, *fpotr;     /* V*r (convention of the potential), -dV/dr*r         */
    const double *potb, *fpotb;     /* rho(r), -drho/dr                                     */
    int           nembd, nkind1;
    double        rhod;             /* RHOD: F(rho) table spacing                           */
    const double *fembd, *dfembd;   /* F(rho), dF/drho at rho = (i-1)*RHOD                  */
    int           ngroup;           /* atom types                                           */
    const int    *kpair;            /* KPAIR(NGROUP,NGROUP), 1-based table ids              */
    const int    *kembd;            /* KEMBD(NGROUP), 1-based (EAM only)                    */
    double        ru;               /* force cutoff RU (the passes use RU^2 = max RU^2)     */
} msmgb_forcetable;

/* One periodic (or not) orthorhombic box of a batch (SimMDBox BOXLOW, ZL; CtrlParam IFPD). */
typedef struct {
    int    natom;
    double lo[3];
    double len[3];
    int    ifpd[3];
} msmgb_box;

/* ---- context ------------------------------------------------------------------------- */
/* Allocates all device memory for the given capacities (replaces Initialize_DEVICES +
 * Allocate_Working_Variables, MD_Globle_Variables_GPU.F90:767-857). */
int  msmgb_create(msmgb_ctx **ctx, const msmgb_params *params);
int  msmgb_destroy(msmgb_ctx *ctx);
const char *msmgb_last_error(const msmgb_ctx *ctx);
void *msmgb_stream(const msmgb_ctx *ctx);          /* cudaStream_t of the context */
int  msmgb_set_precision(msmgb_ctx *ctx, int precision);
/* number of kernels this library has launched on the context so far */
int64_t msmgb_launch_count(const msmgb_ctx *ctx);
int  msmgb_synchronize(msmgb_ctx *ctx);

/* ---- force class (MD_ForceClass_Register_GPU.F90:248-259) ------------------------------ */
/* pIniForcetable: INITIALIZE_FS/EAM_Force_Table_DEV (MD_FS_ForceTable_GPU.F90:178-257,
 * MD_EAM_ForceTable_GPU.F90:192-278): copies the host tables to the device. */
int  msmgb_init_forcetable(msmgb_ctx *ctx, const msmgb_forcetable *ft);
/* pClrForcetable: CLEAR_FS/EAM_Force_Table_DEV */
int  msmgb_clear_forcetable(msmgb_ctx *ctx);
/* pCalForce: CALFORCE_FS/EAM_Force_Table2A_DEV (MD_FS_ForceTable_GPU.F90:934-994,
 * MD_EAM_ForceTable_GPU.F90:950-1010): density pass, F'(rho), force pass. */
int  msmgb_calforce(msmgb_ctx *ctx);
/* pCalPTensor: CALPTENSOR_*_Force_Table2A_DEV (MD_FS_ForceTable_GPU.F90:1348-1411):
 * forces plus the 3x3 virial of every box; vtensor receives 9*nbox values (row-major per
 * box), NOT divided by the number of boxes as the reference's copy-out does (:1462-1463). */
int  msmgb_calptensor(msmgb_ctx *ctx, double *vtensor);
/* pCalEpot: CALEPOT_*_Force_Table2A_DEV (MD_FS_ForceTable_GPU.F90:1720-1742): per-atom
 * potential energy, kept on the device (msmgb_copyout_epot). */
int  msmgb_calepot(msmgb_ctx *ctx);
/* pCalEDen: CALDEN_*_Force_Table2A_DEV (MD_FS_ForceTable_GPU.F90:875-930): F'(rho) only */
int  msmgb_calden(msmgb_ctx *ctx);
/* pCalAVStress: Cal_FS/EAM_AtomicStressTensor_DEV (MD_FS_ForceTable_GPU.F90:2044-2076,
 * MD_EAM_ForceTable_GPU.F90:2073-2106; kernels :1746-1965 / :1775-1994): per-atom virial
 * tensor AP_i(a,b) = sum_j FORTOT s_a s_b (cubic boxes; zero on inactive atoms).  Unlike the
 * reference, which reads the F'(rho) of an earlier force call, this runs its own FP64
 * density pass first.  ap receives 9 slabs of N doubles, component 3a+b (the reference's
 * AP(NAPDEV, 9) layout), in the caller's order (MSMGB_ORDER_ORIGINAL) or sorted order. */
int  msmgb_cal_atomic_stress(msmgb_ctx *ctx, double *ap, int order);

/* ---- state transfer (MD_Globle_Variables_GPU.F90 CopyIn/CopyOut_SimBox_DEV) -------------- */
/* Uploads a batch of boxes (nbox >= 1, boxes concatenated in order).  xp and xp1 are
 * 3*N arrays in XP(N,3) column-major layout; xp1 (velocities) may be NULL (zero).
 * Invalidates the neighbour list. */
int  msmgb_copyin_simbox(msmgb_ctx *ctx, int nbox, const msmgb_box *boxes, const int *ityp,
                         const int *statu, const double *xp, const double *xp1);
/* masses CM(NGROUP) per atom type */
int  msmgb_set_masses(msmgb_ctx *ctx, int ngroup, const double *cm);
/* New positions for the atoms already loaded (XP(N,3), caller order; host or device memory),
 * as a minimiser or saddle search moves them: types, status, velocities and boxes stay;
 * periodic directions are wrapped into the box; the neighbour list is kept while no atom has
 * moved more than the skin trigger since the last build.  Replaces CopyXPFrom_Host_to_Devices
 * (MDLIB/sor/CommonGPU/MD_Globle_Variables_GPU.F90:349-353,2044), which the ART driver calls after
 * moving XP on the host (MDLIB/sor/Appshell/MD_Method_ART_GPU.F90:630). */
int  msmgb_update_positions(msmgb_ctx *ctx, const double *xp);
/* any pointer may be NULL; order = MSMGB_ORDER_ORIGINAL or MSMGB_ORDER_SORTED.  The
 * destination arrays of the copy-out calls may be host or device memory. */
int  msmgb_copyout_simbox(msmgb_ctx *ctx, double *xp, double *xp1, int *statu, double *dis,
                          int order);
int  msmgb_copyout_force(msmgb_ctx *ctx, double *fp, int order);       /* CALEKIN_DEV (MD_DiffScheme_GPU.F90:851-902, copied out in caller order as dbgEKIN): per-atom
 * kinetic energy 0.5 m v^2, -1e32 for an inactive atom or one with a fixed position
 * component; ekin (N) in host or device memory, order MSMGB_ORDER_ORIGINAL or _SORTED. */
int  msmgb_calekin(msmgb_ctx *ctx, double *ekin, int order);
/* FP(N,3)          */
int  msmgb_copyout_epot(msmgb_ctx *ctx, double *epot, int order);     /* EPOT(N)          */
int  msmgb_copyout_den(msmgb_ctx *ctx, double *den, int order);       /* F'(rho_i)        */
/* sorted position -> original index map (hm_GID), N ints */
int  msmgb_copyout_gid(msmgb_ctx *ctx, int *gid);

/* ---- neighbour list (MD_NeighborsList_GPU.F90) --------------------------------------- */
/* Cal_NeighBoreList_DEV (:2316-2372 -> Cal_NeighBoreList2C_0_DEV :1347-1732): cell-sorts
 * the atoms on the device and builds the full list with the FP64 rule d^2 < rc_nl^2. */
int  msmgb_cal_neighborelist(msmgb_ctx *ctx);
/* Copyout_NeighboreList (:718-737): KVOIS(N) and INDI(ld, mxkvois) column-major, 0-based
 * neighbour ids; with MSMGB_ORDER_ORIGINAL both atoms and ids are in the caller's order. */
int  msmgb_copyout_neighborelist(msmgb_ctx *ctx, int *kvois, int *indi, int ld, int order);

/* ---- integrator (MD_DiffScheme_GPU.F90) ------------------------------------------------- */
/* Predictor_DEV (:604-682): x += h v + h^2/2 F/m with PBC wrap, DIS += dx, v += h/2 F/m */
int  msmgb_predictor(msmgb_ctx *ctx, double h);
/* Correction_DEV (:821-848): v += h/2 F/m */
int  msmgb_correction(msmgb_ctx *ctx, double h);
/* For_One_Step (MD_Method_GenericMD_GPU.F90:496-659) repeated nsteps times: predictor,
 * list rebuild when the skin trigger fires (or every NB_UPTAB steps), force, corrector.
 * The steps run as one CUDA graph per step with the rebuild predicated on the device.
 * rebuilds (may be NULL) receives the number of list rebuilds done. */
int  msmgb_run_steps(msmgb_ctx *ctx, int nsteps, double h, int *rebuilds);
/* The same steps split for timing loops: msmgb_enqueue_steps issues nsteps step graphs on
 * the context stream and returns without synchronising; msmgb_finish_steps applies the
 * pending corrector, synchronises and reports errors and the rebuild count since the last
 * finish.  No counterpart in the reference. */
int  msmgb_enqueue_steps(msmgb_ctx *ctx, int nsteps, double h);
int  msmgb_finish_steps(msmgb_ctx *ctx, double h, int *rebuilds);
/* Runs nsteps like msmgb_run_steps and reports the device time of the steps (CUDA events
 * on the context stream, synchronised on both sides) in *ms.  No counterpart in the
 * reference (it times with host CPU_TIME, MD_Method_GenericMD_GPU.F90:246). */
int  msmgb_time_steps(msmgb_ctx *ctx, int nsteps, double h, float *ms, int *rebuilds);
/* Average device time (ms) of one launch of each pass over `reps` launches (out has 5
 * entries): out[0] density pass, out[1] force pass, out[2] list rebuild, out[3] integrator,
 * out[4] fused mixed force pass + integrator (0 when not in use); the integrator kernels are
 * timed with h = 0, which leaves the state unchanged.  No counterpart in the reference. */
int  msmgb_time_passes(msmgb_ctx *ctx, int reps, float *out);
/* Variants picked by the autotuner for the mixed passes (3 entries each): out[0] density
 * pass, out[1] force pass, out[2] fused force pass + integrator; ms (may be NULL) their
 * time per launch.  Tuning runs at the first mixed force call / step graph for a given
 * atom count. */
int  msmgb_get_tuning(const msmgb_ctx *ctx, int *out, float *ms);
/* Number of MD steps captured into one CUDA graph (1..64, default 1): msmgb_run_steps and
 * msmgb_enqueue_steps then launch one graph per k steps (the rest one per step), each step
 * keeping its own device-decided rebuild; the step graphs are rebuilt at the next call.  Fewer
 * host launches per step for small systems and batches of small boxes.  No counterpart in the
 * reference (it launches every kernel of a step from the host, MD_Method_GenericMD_GPU.F90:596-627). */
int  msmgb_set_steps_per_graph(msmgb_ctx *ctx, int k);
/* Graph launches issued by MD steps since the context was created. */
int  msmgb_graph_launch_count(const msmgb_ctx *ctx, int64_t *n);
/* Pins the kernel variants of the mixed passes (codes as returned by msmgb_get_tuning:
 * codes[0] density, codes[1] force, codes[2] fused step kernel; a negative code leaves that
 * choice to the tuner).  Pinned choices are kept for the context's atom count and skip the
 * tuning runs; the step graphs are recaptured.  No counterpart in the reference. */
int  msmgb_set_tuning(msmgb_ctx *ctx, const int *codes);
/* Two-level neighbour list: a full rebuild (cell binning, sort, 27-cell scan) also keeps, per
 * atom, the candidates within rc_nl + skin; later rebuilds re-select the list from them with
 * the same exact rule (the lists are the same sets) until the displacement since the full
 * rebuild may exceed skin/2.  Cells are then sized by rc_nl + skin.  skin = 0 turns it off
 * (every rebuild is full, cells sized by rc_nl as MD_NeighborsList_GPU.F90:289-292); the
 * default is 1.0 A.  A new value applies from the next msmgb_copyin_simbox.  No counterpart
 * in the reference (it rebuilds at a fixed interval, MD_Method_GenericMD_GPU.F90:599). */
int  msmgb_set_outer_skin(msmgb_ctx *ctx, double skin);
/* Non-cubic box: BOXSHAPE of box ibox (SimBox%BOXSHAPE, MD_TypeDef_SimBox.F90:46), row K in
 * bs[3K..3K+2]; the separation of two atoms in length units is BOXSHAPE . SEP, SEP the
 * minimum-image difference of their positions (MD_FS_ForceTable.F90:235,333,
 * MD_NeighborsList.F90:362-364).  Applies from the next msmgb_copyin_simbox; the identity is
 * the default.  A state with a non-identity shape supports the FP64 calls (neighbour list,
 * force, virial, energy, density, per-atom stress); MD, the mixed and float-float passes,
 * the HVP and the adjoint return MSMGB_ERR_ARG for it.  Unlike the reference's GPU force
 * pass (MD_FS_ForceTable_GPU.F90:775), the force pass applies the shape as its density pass
 * and the reference's CPU force routine do. */
int  msmgb_set_boxshape(msmgb_ctx *ctx, int ibox, const double *bs);
/* Device time (ms) of a full list rebuild and of a re-selection from the candidates (0 without
 * a two-level list), averaged over reps launches.  No counterpart in the reference. */
int  msmgb_time_rebuilds(msmgb_ctx *ctx, int reps, float *full_ms, float *inner_ms);
/* List rebuilds done inside MD steps since the context was created, and how many of them
 * were full rebuilds (all of them without a two-level list). */
int  msmgb_rebuild_counts(const msmgb_ctx *ctx, int64_t *rebuilds, int64_t *full);
/* Failure-path self-test of the bounded device waits (the TMA-streamed step kernel's
 * mbarrier waits give up after 0.5 s): runs one block that waits on a barrier nothing
 * completes and returns MSMGB_ERR_TIMEOUT; the context stays usable.  No counterpart in the
 * reference. */
int  msmgb_selftest_wait(msmgb_ctx *ctx);
/* Largest and mean neighbour count of the current list. */
int  msmgb_list_stats(msmgb_ctx *ctx, int *maxk, double *meank);
/* Check of the float-float position records (hi + lo, the list's and the reduced-precision
 * passes' copy of the positions) against the FP64 positions, for every active atom: hi a
 * multiple of the positions' quantum q, |lo| <= q/2, and |hi + lo - (x - lo_box + L)|.
 * *max_err receives the largest of the last in units of q, *violations the number of atoms
 * that break one of the first two.  Diagnostics; no counterpart in the reference. */
int  msmgb_check_records(msmgb_ctx *ctx, double *max_err, int *violations);
/* Cell tiles of the mixed passes for the current list (built after each list build while a
 * selected variant reads them): blocks of 256 sorted atoms, blocks with a tile (a halo of at
 * most 8192 atoms in at most 256 runs), mean and largest halo size over those.  All zero
 * when no tiles are built.  No counterpart in the reference. */
int  msmgb_tile_stats(msmgb_ctx *ctx, int *blocks, int *tiled, double *mean_halo, int *max_halo);

/* ---- external forces (AddExtForce_ForceClass0 / ClearExtForce_ForceClass0 and
 *      Cumulate_ExtForce0, MD_ForceClass_Register_GPU.F90:584-606, 636-656, 982-1180) -------- */
/* What an external-force routine sees: the context's stream, the atoms in the library's
 * sorted device order and the force arrays to add to.  All pointers are device memory. */
typedef struct {
    int           n;          /* atoms                                                        */
    int           nbox;       /* boxes                                                        */
    void         *stream;     /* cudaStream_t: enqueue the work here, do not synchronise      */
    const double *pos;        /* positions, 4 doubles per atom (x, y, z, unused)              */
    double       *fx, *fy, *fz;   /* forces of the force pass just done: add to them          */
    const int    *gid;        /* caller (original) index of each sorted atom                  */
    const int    *ityp, *statu, *boxid;
} msmgb_extforce_view;
/* An external force routine (the reference's pForce procedure of an MDExtForceList entry):
 * returns 0, or a nonzero code that fails the force call with MSMGB_ERR_ARG. */
typedef int (*msmgb_extforce_fn)(void *user, const msmgb_extforce_view *view);
/* Registers fn (with its tag and user pointer) to run after every force pass, in the order of
 * registration, as Calforce_ForceClass0 runs Cumulate_ExtForce0 after pCalForce.  Inside MD
 * steps the step runs unfused (integrator, density pass, force pass, external forces) and is
 * a CUDA graph: fn is called while the step graph is built, so the device work it enqueues
 * on view->stream is replayed every step; its pointers must stay valid and it must not
 * synchronise.  HVP and adjoint calls add no external forces. */
int  msmgb_add_extforce(msmgb_ctx *ctx, const char *tag, msmgb_extforce_fn fn, void *user);
/* ClearExtForce_ForceClass0: removes every registered routine and the field below. */
int  msmgb_clear_extforce(msmgb_ctx *ctx);
/* A constant external force per atom, fext = XP(N,3) layout in the caller's order (host or
 * device memory, copied), added to every active atom after each force pass (a built-in
 * external-force routine: fields, springs held fixed over a run, boosts); NULL removes it.
 * It applies to the current atom count; a copy-in with a different count removes it. */
int  msmgb_set_extforce_field(msmgb_ctx *ctx, const double *fext);

/* ---- differentiation --------------------------------------------------------------------- */
/* Device time of one Hessian-vector product and of one FP64 force call (density + force
 * pass) on the current state, averaged over reps launches (CUDA events on the context
 * stream).  v: 3*N probe, XP layout, caller order.  No counterpart in the reference. */
int  msmgb_time_hvp(msmgb_ctx *ctx, const double *v, int reps, float *ms_hvp, float *ms_force);
/* Hessian-vector product of the table-mode force (exact derivative of the interpolants):
 * hv = -dF/dx . v.  v and hv are 3*N arrays in XP layout, caller's order, in host or device
 * memory.  The first call allocates the pair buffer that hands each pair's geometry from the
 * first pass to the second: 40 B x MXKVOIS per atom of the context's capacity (5.2 GB for
 * 2,048,000 atoms at MXKVOIS 64), kept until msmgb_destroy; MSMGB_ERR_CUDA if it does not fit.
 * No counterpart in the reference: it replaces finite-difference force pairs
 * (MD_Method_ART_GPU.F90:454-576). */
int  msmgb_hvp(msmgb_ctx *ctx, const double *v, double *hv);

/* Force-matching adjoint for the Cleri-Rosato parameters theta = (A, xi, p, q, r0) of the
 * tables currently loaded (which must have been generated from prm): computes the FP64
 * forces F of every box, L = sum_i |F_i - Ft_i|^2 and dL/dtheta (grad[5]) by one adjoint
 * pass pair (density recomputed).  ft: 3*N target forces, XP layout, caller order.
 * No counterpart in the reference (it has no potential fitting). */
int  msmgb_param_adjoint(msmgb_ctx *ctx, int pot, const double *prm, const double *ft,
                         double *loss, double *grad);
/* Parameter derivatives of the Cleri-Rosato tables on the sqrt(r) grid of
 * msmgb_create_forcetable: d[(m*3 + t)*ntab + i-1] for theta_m, m = 0..4, and t = 0 FPOTR,
 * 1 POTB, 2 FPOTB.  Host only. */
int  msmgb_cr_param_tables(const double *prm, double rmax, int ntab, double *d);

/* ---- force call without device allocation ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot let this library call cudaMalloc:
 * a host code whose device arrays are already owned by its own runtime (such as msmpscu's
 * CUDA Fortran work arrays), a code held to a fixed device-memory budget by its own
 * allocator, or one that must not let cudaMalloc's implicit device synchronisation stall its
 * other streams mid-step.  The caller passes device pointers to all inputs and the output;
 * the only extra memory, F'(rho) of every atom between the two passes plus one error word,
 * sits in a fixed array compiled into the library (8 MiB per GPU, held until exit), so at
 * most MSMGB_NOALLOC_MAX_ATOMS atoms can be handled (larger n returns MSMGB_ERR_CAPACITY).
 * The first call on a device, made with that device current, looks up the device address of
 * that array; under CUDA's lazy module loading (the default) that first call also loads the
 * library's device code onto the device, which synchronises it, so make this first call at
 * set-up, before any stream capture and before time-critical work.  All calls on a device share
 * the array and it keeps the last call's contents (the error word is cleared at the start of
 * every call); calls whose work overlaps on the GPU race on it, so serialise them.
 * FP64, single species (tables of kind 1), orthorhombic box; the call synchronises `stream`.
 * INDI holds 0-based neighbour ids (the reference's INDI is 1-based: subtract 1 first); an id
 * outside 0..n-1 is not read, its slot is skipped and the call returns MSMGB_ERR_ARG.
 * Results equal msmgb_calforce's to rounding. */
#define MSMGB_NOALLOC_MAX_ATOMS 1048576
typedef struct {
    int           n;          /* atoms (<= MSMGB_NOALLOC_MAX_ATOMS)                          */
    const double *xp;         /* device: XP(N,3) column-major positions                     */
    const int    *statu;      /* device: STATU(N)                                            */
    const int    *kvois;      /* device: KVOIS(N)                                            */
    const int    *indi;       /* device: INDI(ld, *) column-major, 0-based neighbour ids    */
    int           ld;         /* leading dimension of indi (>= n)                           */
    double        box_len[3]; /* box edges                                                  */
    int           ifpd[3];    /* periodic flags                                             */
    int           pottype;    /* MSMGB_FS_TYPE or MSMGB_EAM_TYPE                            */
    int           ntab;       /* pair table points                                          */
    double        rmax;       /* table Rmax                                                 */
    double        ru;         /* force cutoff                                               */
    const double *potb, *fpotr, *fpotb;   /* device: NTAB entries each (reference layout)   */
    int           nembd;      /* EAM: F'(rho) table points                                  */
    double        rhod;       /* EAM: F'(rho) table spacing                                 */
    const double *dfembd;     /* EAM, device: NEMBD entries                                 */
    double       *fp;         /* device output: FP(N,3) column-major forces                 */
    void         *stream;     /* cudaStream_t (NULL: legacy default stream)                 */
    char         *errbuf;     /* optional host buffer for an error message                  */
    int           errlen;
} msmgb_force_noalloc;
int  msmgb_calforce_noalloc(const msmgb_force_noalloc *args);

/* ---- host-side table generator (Create_Interaction_ForceTable,
 *      MD_TypeDef_ForceTable.F90:890-1056) -------------------------------------------------- */
#define MSMGB_POT_CR          1   /* Cleri-Rosato TB-SMA, FS form; prm = A, xi, p, q, r0     */
#define MSMGB_POT_MARINICA2   2   /* Marinica EAM2 for W (EAM form); prm unused              */
#define MSMGB_POT_ACKLAND_WW  3   /* Ackland-Thetford W, FS form; prm unused                 */
/* the rest of the W-He library EM_TB_WangJun_W-HE_2010 (EM_TB_ForceTable_WangJun_W_HE_2010.F90:68-121) */
#define MSMGB_POT_DERLET_WW   4   /* Derlet-Nguyen-Manh-Dudarev W, FS form (FS_PM_WW.F90)      */
#define MSMGB_POT_HEHE_EXP6   5   /* He-He ZBL / cubic / EXP6, no density (ZBL_EXP6_HeHe.F90)  */
#define MSMGB_POT_HEW_ZBL     6   /* He-W ZBL / cubics / EXP6, no density (ZBL_ABINTIO_He_W_930.F90) */
/* the other subtypes of EAM_WW_Marinica_JPCM25_2013 (EAM_ForceTable_Marinica_JPCM25_2013.F90:31-44) */
#define MSMGB_POT_MARINICA3   7   /* Marinica EAM3 for W (EAM form); prm unused              */
#define MSMGB_POT_MARINICA4   8   /* Marinica EAM4 for W (EAM form); prm unused              */
/* EM_TB_Ackland_Vitek_PRB41_10324 (EM_TB_ForceTable_Ackland_Vitek_PRB41_10324.F90), FS form */
#define MSMGB_POT_AV_CU       9   /* Cu-Cu                                                   */
#define MSMGB_POT_AV_AU      10   /* Au-Au                                                   */
#define MSMGB_POT_AV_CUAU    11   /* Cu-Au cross pair and density sqrt(rho_Cu rho_Au)        */
#define MSMGB_POT_MENDELEV_ZR 12  /* Mendelev-Ackland Zr, EAM form (EAM_ZrZr_Mendelev_Phil_Mag_L87_2007.F90) */
#define MSMGB_POT_AWB_ZR     13   /* Ackland-Wooding-Bacon Zr, FS form (EM_TB_AWB_Phil_Mag_A71_1995_553.F90) */
#define MSMGB_POT_HETI_LJ    14   /* He-Ti pair, no density (EM_TB_WangJun_Ti-HE_2007/LJ_He_Ti.F90) */
/* Fills POTR/FPOTR/POTB/FPOTB (ntab each) and, if fembd/dfembd are non-NULL, F/F' (nembd
 * each); returns RHOD = rhoscal * max(POTB) / nembd through *rhod.  Lengths in Angstrom,
 * energies in eV. */
int  msmgb_create_forcetable(int pot, const double *prm, double rmax, int ntab, int nembd,
                             double rhoscal, double *potr, double *fpotr, double *potb,
                             double *fpotb, double *fembd, double *dfembd, double *rhod);

/* ---- tabulated EAM potentials in setfl layout (Register_ForceTableProc_Setfl,
 *      Filedatas_Func_Setfl.F90:499-541; reader get_filedatas_setfl :119-253) ------------- */
/* Element count, grid sizes and cutoff of a setfl file (Angstrom / eV, LAMMPS layout). */
int  msmgb_setfl_info(const char *path, int *nelem, int *nrho, int *nr, double *cutoff);
/* Tables of a setfl file on the sqrt(r) grid of ntab points up to Rmax = cutoff, EAM type:
 * NKIND = NE^2 pair tables (id (I-1)*NE + J for an I atom with a J neighbour: the pair
 * phi_IJ and the density of element J) in the (NKIND, NTAB) column-major layout of
 * msmgb_forcetable with POTR = 0.5 r phi, FPOTR = -r phi', POTB = rho_J, FPOTB = -rho_J';
 * NKIND1 = NE embedding tables F, F' on the file's rho grid (NEMBD = Nrho, RHOD = drho),
 * (NKIND1, NEMBD) column-major; KPAIR (NE, NE) column-major, KEMBD (NE), masses (NE, amu).
 * Interpolation: natural cubic spline through the file's data (the reference's SLATEC
 * DBINT4/DBVALU settings, :25-34, 256-276).  Host only. */
int  msmgb_setfl_tables(const char *path, int ntab, double *potr, double *fpotr, double *potb,
                        double *fpotb, double *fembd, double *dfembd, int *kpair, int *kembd,
                        double *rhod, double *masses);

/* ---- Bonny, Grigorev, Terentyev W-H-He EAM (EAM_WHeH_Bonny_JPCM26_2014;
 *      EAM_ForceTable_Bonny_JPCM26_2014.F90:17-121) ---------------------------------------- */
/* subtype 1 = EAM1 (H and He pair-only), 2 = EAM2 (H embedded in the W density).  Writes
 * *nkind = 9 (EAM1) or 10 (EAM2, table #10 zero) tables in the reference's registration order,
 * (NKIND, NTAB) column-major (caller allocates 10*ntab), on the sqrt(r) grid up to rmax; the
 * embedding tables of W, H, He (3, NEMBD) column-major with RHOD = rhoscal * max POTB / nembd
 * (rhoscal <= 0: 20); KPAIR (3,3) column-major for groups W = 1, H = 2, He = 3 with the host
 * first, KEMBD = 1, 2, 3.  Host only. */
int  msmgb_bonny_wheh_tables(int subtype, double rmax, int ntab, int nembd, double rhoscal,
                             double *potr, double *fpotr, double *potb, double *fpotb, double *fembd,
                             double *dfembd, int *kpair, int *kembd, int *nkind, double *rhod);

/* ---- Moldy potential files (Register_ForceTableProc_Moldy,
 *      MDLIB/sor/Potentials/EAM_NIST/Filedatas_Func_Moldy.F90:27-77,116-131) ------------------ */
/* One element, EAM type with F = -sqrt(rho): the pair and density knot sums of the file
 * (knots times the lattice constant a0, coefficients over a0^3 and a0^6) on the sqrt(r) grid of
 * ntab points up to rmax (the cutoff), the embedding table of nembd points on
 * RHOD = rhoscal * max POTB / nembd (rhoscal <= 0: 20).  Host only. */
int  msmgb_moldy_tables(const char *path, double rmax, int ntab, int nembd, double rhoscal,
                        double *potr, double *fpotr, double *potb, double *fpotb, double *fembd,
                        double *dfembd, double *rhod);

/* ---- tabulated EAM potentials in lspt layout (Register_ForceTableProc_SPT,
 *      MDLIB/sor/Potentials/EAM_NIST/Filedatas_Func_Lspt.F90:560-604; reader
 *      get_filedatas_lspt :118-301) ------------------------------------------------------- */
/* flags: the reference reads the first file named on each pair line for every pair of that
 * line (:263); MSMGB_LSPT_EACH_VR_FILE reads each named file instead. */
#define MSMGB_LSPT_EACH_VR_FILE 1
/* Element count, largest pair-file r (Angstrom) and largest F(rho)-file rho of an lspt
 * control file and the ".spt" files it names. */
int  msmgb_lspt_info(const char *path, int flags, int *nelem, double *rmax, double *rhomax);
/* Tables of an lspt potential, EAM type, in the layouts of msmgb_setfl_tables: NKIND = NE^2
 * pair tables on the sqrt(r) grid of ntab points up to rmax (<= 0: the files' largest r, the
 * reader's RMAX), POTR = 0.5 V r, FPOTR = -V' r, POTB = rho_J, FPOTB = -rho_J'; NKIND1 = NE
 * embedding tables of nembd points, RHOD = largest F(rho)-file rho / nembd (the reader's RHOMX,
 * which the NIST generator keeps, NIST_ForceTable.F90:379-413).  Natural cubic splines through
 * the data with the reader's range rules (Vr_Spline, Rhor_Spline, Frho_Spline :340-500).
 * Host only.  Returns MSMGB_ERR_ARG for a missing or malformed file. */
int  msmgb_lspt_tables(const char *path, int flags, int ntab, int nembd, double rmax,
                       double *potr, double *fpotr, double *potb, double *fpotb, double *fembd,
                       double *dfembd, int *kpair, int *kembd, double *rhod);

/* ---- tables exported by the reference and read back (Import_ForceTable,
 *      Register_Imported_ForceTable, Export_ForceTable; MD_TypeDef_ForceTable.F90:1315-1855) ---- */
/* Units of the tables these calls return or take: the files are in Angstrom / eV;
 * MSMGB_UNITS_CGS applies the reference's conversions on import (:1529-1540, 1583-1585) so the
 * tables match its CGS force table (lengths in cm, energies in erg, FS densities in erg^2). */
#define MSMGB_UNITS_EV_A 0
#define MSMGB_UNITS_CGS  1
/* Header of stem.pair / stem.embd: potential type, table ids (FPAIR, up to 256) and grid
 * sizes of both files.  Host only.  Returns MSMGB_ERR_ARG for a missing or malformed file. */
int  msmgb_import_info(const char *stem, int *pottype, int *ntables, int *ids, int *npoint,
                       int *nembtables, int *emb_ids, int *nembpoint);
/* Register_Imported_ForceTable (:1612-1855) for a box of ngroup atom types whose pairs use
 * the file tables PTYPE(NGROUP,NGROUP) (column-major, ids as in the files): the tables named
 * are numbered by first appearance (KPAIR, KEMBD as New_ForceTable :560-574, 600-610) and
 * re-gridded by the reference's spline (SPLID1/SPLID2 with end slopes from the four end rows,
 * LIB/sor/f/MiniUtilities/DINTF2.F:17-240) onto the sqrt(r) grid of ntab points up to rmax
 * (0 beyond the file's largest r) and, for EAM, onto rho = (i-1)*RHOD with RHOD = RHOMX/nembd,
 * RHOMX = RHO(N)*N/(N-1) of the file's N embedding rows.  Outputs in the (NKIND, NTAB) /
 * (NKIND1, NEMBD) column-major layouts of msmgb_forcetable (caller allocates ngroup^2*ntab and
 * ngroup*nembd); kpair (ngroup^2), kembd (ngroup, EAM only), *nkind, *nkind1 (0 for FS),
 * *rhod, *pottype.  rmax, tables and RHOD in `units`.  Host only.  MSMGB_ERR_ARG for a
 * missing file or a PTYPE id absent from either file (the reference stops there). */
int  msmgb_import_forcetable(const char *stem, int units, int ngroup, const int *ptype, double rmax,
                             int ntab, int nembd, double *potr, double *fpotr, double *potb,
                             double *fpotb, double *fembd, double *dfembd, int *kpair, int *kembd,
                             int *nkind, int *nkind1, double *rhod, int *pottype);
/* Export_ForceTable (:1315-1459): writes stem.pair and stem.embd in the reference's layout
 * (rows 1PE21.9 / 1PE16.8, tables in increasing id order) from the tables of ft (in `units`);
 * ids / emb_ids name the NKIND pair and NKIND1 embedding tables (NULL: 1, 2, ...).  An FS
 * table gets the reference's informational embedding file (F = -sqrt(rho) on RHOD).  Host only. */
int  msmgb_export_forcetable(const char *stem, int units, const msmgb_forcetable *ft, const int *ids,
                             const int *emb_ids);

#ifdef __cplusplus
}
#endif
#endif
