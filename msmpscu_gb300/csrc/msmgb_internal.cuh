// msmgb_internal.cuh -- device data layout and kernel entry points shared by the
// translation units of libmsmgb.so.  Not part of the public ABI.
//
// Layout in HBM (all per-atom arrays are in cell-sorted order, capacity = max_atoms):
//   pos      double4_32a  x, y, z, (unused)           gathered by the pair loops (one 32 B sector)
//   posff    2xfloat4 float-float copy of the position in the shifted frame u = x - lo + L
//                     (u in [L, 2L], so hi_i - hi_j is exact); rebuilt by the integrator,
//                     gathered by the list prefilter and the mixed passes
//   vx..vz   double   velocities (SoA, streamed)
//   fx..fz   double   forces (SoA, streamed)
//   dis      double   accumulated displacement DIS (reference MD_DiffScheme_GPU.F90:364-366)
//   pos_bld  float4   FP32 shifted positions (hi + lo) at the last list build (skin
//                     trigger and list-build candidates; differences are exact)
//   ityp, statu, gid (sorted -> original), boxid
//   kvois    int32    neighbour count, INDI column-major int32 [mxkvois][cap] (reference
//                     layout INDI(NAPDEV,MXKVOIS), MD_NeighborsList_GPU.F90:75-85)
//   tables   double   per kind, NTAB+2 entries (index 0 and NTAB+1 padded: the reference reads NTAB+1 when r = Rmax)
#pragma once
#include <cuda.h>            // CUtensorMap (type only; the encoder is fetched at run time)
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/msmgb.h"

#include <nvtx3/nvToolsExt.h>

namespace msmgb {

// NVTX range around an entry point of the C ABI (seen by nsys / ncu range filters; costs a
// function-pointer test when no profiler is attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

constexpr int kBlock = 256;
constexpr int kMaxGroups = 16;          // mp_MXGROUP, MD_Const.F90:77
// longest edge span (the edge, or twice an open edge) of the fixed-point force records: a unit
// of at most 2.4e-7 A
constexpr double kFixMaxSpan = 1024.0;

// cell tiles (k_halo): a block of kBlock sorted atoms spanning at most kHaloCells cells,
// whose halo has at most kHaloRuns runs and kHaloMax atoms, gets a tile; others none
constexpr int kHaloCells = 64;
constexpr int kHaloRuns = 256;
constexpr int kHaloMax = 8192;

// error bits in flags[kFlagErr]
constexpr int kErrOverflow = 1;
constexpr int kErrOutOfBox = 2;
constexpr int kErrRho = 4;
constexpr int kErrTimeout = 8;
constexpr int kErrNonFinite = 16;   // a position that is not a finite number
constexpr int kErrBadList = 32;     // list validation (MSMGB_CHECK_LISTS=1) found a bad entry
constexpr int kErrCandOverflow = 64;  // an atom has more candidates than the candidate list holds

// device flag words
enum {
    kFlagErr = 0,        // error bits
    kFlagRebuild = 1,    // 1: the list is rebuilt in this step
    kFlagRebuilds = 2,   // number of rebuilds done by run_steps
    kFlagPending = 3,    // 1: a corrector half-kick is pending (fused integrator)
    kFlagStep = 4,       // step counter for the fixed-interval rebuild
    kFlagMaxK = 5,       // largest neighbour count seen by the last build
    kFlagFull = 6,       // number of full rebuilds (two-level list) done by run_steps
    kFlagAcc = 7,        // float bits: bound on the displacement since the last full rebuild
    kFlagOob = 8,        // an atom left its box since the last full rebuild (next one is full)
    kFlagMaxCand = 9,    // largest candidate count of the last full rebuild (two-level list)
    kFlagFullNow = 10,   // 1: this step's rebuild is full (two-level list, read by k_set_full)
    kFlagWords = 16
};

// float-float position (hi, lo parts of u = x + ushift).  In the record buffer `rec` the
// mixed density pass writes d = the atom's FP32 F'(rho) next to its position, so the force
// pass gets a neighbour's position and F'(rho) with one 32 B gather.
struct __align__(32) PosFF {
    float hx, hy, hz, d;
    float lx, ly, lz, lw;
};

// Position record of the float-float passes: hi = float(u) of u = x + ushift and the exact
// remainder u - hi as an integer multiple of the box's quantum (fxq = 2^-30 of the largest
// ulp of hi), so separations and image shifts are exact integer differences; dh, dl carry
// F'(rho) in the records written by the float-float density pass.
struct __align__(32) PosFX {
    float hx, hy, hz;
    int qx, qy, qz;
    float dh, dl;
};

struct DevBox {
    double lo[3];
    double len[3];
    double half[3];
    double ushift[3];    // L - lo: u = x + ushift is the float-float frame coordinate
    double ushs[3];      // ushift 2^S, 2^S = pscale = 2^32 / qq (make_posff)
    double pscale;
    float plo;           // 2^-S
    long long klo[3], kub[3];   // order-preserving integer keys of lo and lo + L
    float lenf[3];       // float-float box length (hi, lo) and FP32 half length
    float lenlo[3];
    float halff[3];
    float dlmax;         // bound on the low part of a float-float separation component (posff)
    float dlfx;          // the same for the integer-remainder records of the float-float passes
    // hi parts of the float-float positions are multiples of the quantum qq (a power of two):
    // hi differences and their squares are exact in FP32 for pairs below ~18 A; qmag =
    // 1.5 2^23 qq rounds a hi value to the quantum by one add and one subtract
    float qq, qmag;
    float fxq;           // float-float passes: quantum of the integer remainders (power of 2)
    double fxinv;        // 1 / fxq
    // fixed-point records of the mixed force passes: coordinate k as (x - lo) / fixu[k] mod 2^32,
    // fixu[k] = L_k / 2^32 on a periodic edge (the wrapping int32 difference is the minimum
    // image) or 2 L_k / 2^32 on an open one.  From a float-float position (hi a multiple of the
    // quantum qq): x - lo = m qq + r with m = (hi - fixlq) / qq an integer and r = lo - fixll
    // (fixlq: L rounded to qq, fixll = L - fixlq), and (x - lo) / unit = m fixa 2^-32 + r fixs,
    // fixa = round(qq / unit 2^32), fixs = 1 / unit
    float fixu[3];
    float fixlq[3], fixll[3], fixs[3];
    unsigned long long fixa[3];
    float qinv;          // 1 / qq
    double bs[9];        // BOXSHAPE(K, 1:3) in row K: separations in length units are bs . SEP
    int shaped;          // bs is not the identity (FP64 static calls only)
    int lq[3];           // (L - float(L)) / fxq, exact
    int ifpd[3];
    int nc[3];
    int cell0;           // first global cell id of this box
    int atom0, natom;    // atom range in the caller's (original) order
};

struct DevTables {
    int pottype;
    int ntab, nkind, ntp;          // ntp = ntab + 2 (padded row length)
    double csi, ru2;
    const double *potr, *fpotr, *potb, *fpotb;     // [nkind][ntp]
    // mixed-precision tables: value and slope to the next grid point, interleaved
    const float2 *dens2;           // [nkind][ntp] {POTB(k), POTB(k+1)-POTB(k)}
    const float4 *force4;          // [nkind][ntp] {FPOTR, dFPOTR, FPOTB, dFPOTB}
    const float2 *embd2;           // [nkind1][nep] {DFEMBD, dDFEMBD}
    // float-float tables: {value hi, lo, slope hi, lo} (slope to the next grid point in FP64)
    const float4 *densff;          // [nkind][ntp] POTB
    const float4 *forceff;         // [nkind][ntp][2] FPOTR, FPOTB
    const float4 *embff;           // [nkind1][nep] DFEMBD
    // table-assisted index of the mixed density pass: per kind and grid point k
    // {POTB(k), POTB(k+1) - POTB(k), hi and lo of r2_k = (k/CSI)^4}
    const float4 *densq;           // [nkind][ntp]
    float irhodh, irhodl;          // 1 / RHOD as float-float
    float csih, csil;              // CSI as float-float
    float ru2h, ru2l;              // RU^2 as float-float
    float rhodf;
    int nembd, nkind1, nep;        // nep = nembd + 2
    double rhod;
    const double *fembd, *dfembd;  // [nkind1][nep]
    int ngroup;
    int kpair[kMaxGroups * kMaxGroups];   // 0-based kind for (ityi, ityj): kpair[(ityj)*ng + ityi]
    int kembd[kMaxGroups];
};

// Pointers of the atom state, passed by value to kernels.
struct DevAtoms {
    double4_32a *pos;
    PosFF *posff;
    double4_32a *pos_nxt;    // fused mixed step: positions of step n+1 (second buffer)
    PosFF *posff_nxt;
    double *vx, *vy, *vz;
    double *fx, *fy, *fz;
    double *dx, *dy, *dz;
    float4 *pos_bld;
    int *ityp, *statu, *gid, *boxid;
    double *den, *epot;
    float *den32;
    int *kvois, *indi;
    int ld;              // leading dimension of indi (capacity)
    int mxk;
    int n;
    const DevBox *box;
    const double *cm;    // masses per type (0-based type index)
    const double *icm;   // reciprocal masses per type
    unsigned *pk;        // mixed passes: per-pair table index (KK << 18 | DK * 2^18), ELL layout
    PosFF *rec;          // mixed passes: {position, F'(rho)} records written by the density pass
    // mixed passes: 16 B fixed-point records {x, y, z (DevBox::fixu units), F'(rho) bits}, also
    // written by the density pass when fix_on (every box edge short enough, see fix_record)
    uint4 *rec16;
    int fix_on;
    PosFX *posfx;        // float-float passes: positions (k_fix) ...
    PosFX *recfx;        // ... and {position, F'(rho)} records written by the density pass
    // cell tiles of the mixed passes (k_halo, after each list build): for the 256 atoms of
    // block b, the atoms of every cell in the 27-cell stencils of their cells ("halo") as runs
    // of consecutive sorted atoms; lidx = each list slot's position in the block's halo
    unsigned short *lidx;   // ELL layout like indi
    int2 *hmeta;            // [block] {number of runs, halo atoms}; {-1, 0}: no tile
    int2 *hruns;            // [block][kHaloRuns + 1] {first atom, offset in the halo}
    int *flags;
    unsigned long long *maxdisp;
    double *virial;      // [nbox][6]
};

// Threads per block for the one-thread-per-atom kernels: 256 for large systems, smaller
// blocks when fewer than two blocks per SM (152 SMs) would be launched, so small systems
// (16,001-atom W, 4,000-atom Cu) still spread over every SM.
inline int block_for(int n)
{
    if (n >= 256 * 2 * 152) return 256;
    if (n >= 128 * 2 * 152) return 128;
    return 64;
}

// u = x + ushift = hi + lo with hi the nearest multiple of the box's quantum qq to u and lo the
// rest, through u in fixed point with 2^32 units per quantum: M = rint(u 2^S), 2^S = 2^32 / qq
// (the FMA forms (x + ushift) 2^S, rounded once as x + ushift would be: scaling by a power of
// two commutes with the rounding).  The high word of M + 2^31 is round(u / qq), so hi = that
// times qq (exact in FP32: |u| < 2^23 qq); the low word less 2^31 is the remainder r in
// [-2^31, 2^31) units and lo = float(r) 2^-S, |lo| <= qq/2, within qq (2^-26 + 2^-33) of
// u - hi.  Two FP64-pipe instructions (the FMA and the conversion) instead of the five of a
// split by conversions to FP32 and back.
__device__ __forceinline__ void split_q(double x, double scale, double ushs, float qq, float plo, float &h,
                                        float &l)
{
    // unsigned add: no signed overflow for a saturated conversion of a coordinate far outside
    const unsigned long long m = (unsigned long long)__double2ll_rn(fma(x, scale, ushs)) + 0x80000000ull;
    h = __int2float_rn((int)((long long)m >> 32)) * qq;
    l = __int2float_rn((int)((unsigned)m ^ 0x80000000u)) * plo;
}

__device__ __forceinline__ PosFF make_posff(double x, double y, double z, const DevBox &b)
{
    PosFF p;
    split_q(x, b.pscale, b.ushs[0], b.qq, b.plo, p.hx, p.lx);
    split_q(y, b.pscale, b.ushs[1], b.qq, b.plo, p.hy, p.ly);
    split_q(z, b.pscale, b.ushs[2], b.qq, b.plo, p.hz, p.lz);
    p.d = 0.0f;
    p.lw = 0.0f;
    return p;
}

// One 256-bit load / store per 32 B record (sm_100+ vector width): a gather of 32 lanes'
// records then touches each sector once instead of once per 16 B half.  The records are
// 32 B aligned (PosFF is __align__(32), buffers come from cudaMalloc).
__device__ __forceinline__ PosFF ld_ff(const PosFF *p)
{
    PosFF r;
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.hx), "=f"(r.hy), "=f"(r.hz), "=f"(r.d), "=f"(r.lx), "=f"(r.ly), "=f"(r.lz), "=f"(r.lw)
        : "l"(p));
    return r;
}

__device__ __forceinline__ void st_ff(PosFF *p, const PosFF &r)
{
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(r.hx), "f"(r.hy),
                 "f"(r.hz), "f"(r.d), "f"(r.lx), "f"(r.ly), "f"(r.lz), "f"(r.lw)
                 : "memory");
}

// the position as one FP32 value per component (hi + lo), for the list prefilter and the skin
// trigger: within one ulp of float(u)
__device__ __forceinline__ float4 pos_f32(const PosFF &f)
{
    return make_float4(f.hx + f.lx, f.hy + f.ly, f.hz + f.lz, 0.0f);
}

// 16 B fixed-point record of an atom for the mixed force passes, from its float-float position
// and its F'(rho), in integer and FP32 arithmetic (DevBox::fixa): the whole units come from the
// exact 64-bit product m fixa (taken mod 2^64, so mod 2^32 after the shift), the rest
// (fraction of that product + r / unit, below ~1.2e5 units) in FP32; within one unit of the
// rounded (x - lo) / unit.  With edge spans up to 1,024 A the unit is at most 2.4e-7 A, so a
// separation formed from two records, (float)(int)(q_i - q_j) * unit, carries ~1e-7 of its
// length.
__device__ __forceinline__ uint4 fix_record(const PosFF &p, float d, const DevBox &b)
{
    const float h[3] = {p.hx, p.hy, p.hz}, l[3] = {p.lx, p.ly, p.lz};
    unsigned q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int m = __float2int_rn((h[k] - b.fixlq[k]) * b.qinv);           // exact
        const unsigned long long P = (unsigned long long)(long long)m * b.fixa[k];
        const float fr = __uint2float_rn((unsigned)P) * 2.3283064365386963e-10f;   // 2^-32
        const float f = fmaf(l[k] - b.fixll[k], b.fixs[k], fr);
        q[k] = (unsigned)(P >> 32) + (unsigned)__float2int_rn(f);
    }
    return make_uint4(q[0], q[1], q[2], __float_as_uint(d));
}

// non-cubic box: DXYZ(K) = sum(BOXSHAPE(K,1:3)*SEP(1:3)) after the minimum image
// (MD_FS_ForceTable.F90:235,333; MD_NeighborsList.F90:362-364)
__device__ __forceinline__ void shape_sep(const DevBox &b, double &sx, double &sy, double &sz)
{
    if (!b.shaped) return;
    const double x = sx, y = sy, z = sz;
    sx = b.bs[0] * x + b.bs[1] * y + b.bs[2] * z;
    sy = b.bs[3] * x + b.bs[4] * y + b.bs[5] * z;
    sz = b.bs[6] * x + b.bs[7] * y + b.bs[8] * z;
}

__device__ __forceinline__ float mi32f(float s, float len, float half, int pd)
{
    return (pd && fabsf(s) > half) ? s - copysignf(len, s) : s;
}

// order-preserving integer key of a double: x > y <=> key(x) > key(y)
__device__ __forceinline__ long long okey(double x)
{
    const long long k = __double_as_longlong(x);
    return k ^ ((k >> 63) & 0x7fffffffffffffffLL);
}

// periodic wrap of one new coordinate (x - L above the box, x + L below it; x + (-L) is x - L
// exactly) and the out-of-box flags from its integer key.  Few atoms cross a face in one step:
// the shift sits behind a vote of the lanes running this code, so a warp with no crossing lane
// skips it (if-converted, both shifts ran for every atom).
__device__ __forceinline__ double wrap_coord(double x, int pd, double len, long long klo, long long kub,
                                             int &oob_hi, int &oob_lo)
{
    long long k = okey(x);
    const bool out = pd && (k > kub || k < klo);
    if (__any_sync(__activemask(), out)) {
        if (out) {
            x = x + (k > kub ? -len : len);
            k = okey(x);
        }
    }
    oob_hi |= k > kub;
    oob_lo |= k < klo;
    return x;
}

// one coordinate of Predictor_KERNEL0 (MD_DiffScheme_GPU.F90:314-349): DIS = h v + h^2/2 a
// (0 if FIXPOS), x += DIS, periodic wrap when x > lo + L or x < lo.  The box tests compare
// integer keys (same order as the doubles) so they stay off the FP64 pipe.
__device__ __forceinline__ double advance(double x0, double v, double a, double th, double h2s2, bool fix,
                                          int pd, double len, long long klo, long long kub, double &dis,
                                          int &oob_hi, int &oob_lo)
{
    const double d = fix ? 0.0 : fma(h2s2, a, th * v);
    dis = d;
    return wrap_coord(x0 + d, pd, len, klo, kub, oob_hi, oob_lo);
}

// The same coordinate with the displacement formed from the advanced velocity: vk = v + k F
// (k = the kicks' h/2 or h times 1/m), DIS = h vk.  With k = h/(2m) DIS = h v + h^2/2 F/m as
// above; with k = h/m (the corrector's and the predictor's half kicks by the same force) vk is
// v(n+1/2) and DIS = h v(n) + h^2/2 F/m with v(n) the corrected velocity.  Two FP64
// instructions per component instead of five (F/m, the two kicks, h v, the FMA).  v becomes
// vk unless the component's velocity is fixed.
__device__ __forceinline__ double advance_hv(double x0, double &v, double f, double k, bool fv, double th,
                                             bool fix, int pd, double len, long long klo, long long kub,
                                             double &dis, int &oob_hi, int &oob_lo)
{
    const double vk = fma(k, f, v);
    const double d = fix ? 0.0 : th * vk;
    if (!fv) v = vk;
    dis = d;
    return wrap_coord(x0 + d, pd, len, klo, kub, oob_hi, oob_lo);
}

// Corrector of step n (v += h/2 F/m) followed by the predictor of step n+1 for one active
// atom (Correction_KERNEL :741-749 then Predictor_KERNEL0 :290-378); positions are read from
// pin and written to pout / fout.  Returns the squared displacement since the last build.
// HV (the mixed-precision passes): advance_hv, the same update in fewer FP64 instructions,
// rounded differently (the passes' FP32 forces carry ~1e-7 of the force, far above that);
// the FP64 and float-float passes keep the reference's operation order.  A fixed velocity
// component (FIXVEL or FIXPOS) gets no corrector kick, so its k stays h/(2m).
template <bool HV = false>
__device__ __forceinline__ float vv_atom(const DevAtoms &a, int i, int stat, const DevBox &b, double th,
                                          bool corrector, double fx, double fy, double fz,
                                          const double4_32a &p, double4_32a *pout, PosFF *fout)
{
    const double icm = a.icm[a.ityp[i] - 1];
    double vx = a.vx[i], vy = a.vy[i], vz = a.vz[i];
    const bool fvx = (stat & (MSMGB_STATU_FIXVELX | MSMGB_STATU_FIXPOSX)) != 0;
    const bool fvy = (stat & (MSMGB_STATU_FIXVELY | MSMGB_STATU_FIXPOSY)) != 0;
    const bool fvz = (stat & (MSMGB_STATU_FIXVELZ | MSMGB_STATU_FIXPOSZ)) != 0;
    int hi = 0, lo = 0;
    double dx, dy, dz, x, y, z;
    if constexpr (HV) {
        // (h/m)/2 is (h/2)/m exactly
        const double k1 = th * icm, kf = k1 * 0.5, kv = corrector ? k1 : kf;
        x = advance_hv(p.x, vx, fx, fvx ? kf : kv, fvx, th, (stat & MSMGB_STATU_FIXPOSX) != 0, b.ifpd[0],
                       b.len[0], b.klo[0], b.kub[0], dx, hi, lo);
        y = advance_hv(p.y, vy, fy, fvy ? kf : kv, fvy, th, (stat & MSMGB_STATU_FIXPOSY) != 0, b.ifpd[1],
                       b.len[1], b.klo[1], b.kub[1], dy, hi, lo);
        z = advance_hv(p.z, vz, fz, fvz ? kf : kv, fvz, th, (stat & MSMGB_STATU_FIXPOSZ) != 0, b.ifpd[2],
                       b.len[2], b.klo[2], b.kub[2], dz, hi, lo);
    } else {
        const double hs2 = th * 0.5, h2s2 = th * th * 0.5;
        const double ax = fx * icm, ay = fy * icm, az = fz * icm;
        if (corrector) {
            if (!fvx) vx = fma(hs2, ax, vx);
            if (!fvy) vy = fma(hs2, ay, vy);
            if (!fvz) vz = fma(hs2, az, vz);
        }
        x = advance(p.x, vx, ax, th, h2s2, (stat & MSMGB_STATU_FIXPOSX) != 0, b.ifpd[0], b.len[0],
                    b.klo[0], b.kub[0], dx, hi, lo);
        y = advance(p.y, vy, ay, th, h2s2, (stat & MSMGB_STATU_FIXPOSY) != 0, b.ifpd[1], b.len[1],
                    b.klo[1], b.kub[1], dy, hi, lo);
        z = advance(p.z, vz, az, th, h2s2, (stat & MSMGB_STATU_FIXPOSZ) != 0, b.ifpd[2], b.len[2],
                    b.klo[2], b.kub[2], dz, hi, lo);
        if (!fvx) vx = fma(hs2, ax, vx);
        if (!fvy) vy = fma(hs2, ay, vy);
        if (!fvz) vz = fma(hs2, az, vz);
    }
    pout[i] = make_double4_32a(x, y, z, p.w);
    const PosFF f = make_posff(x, y, z, b);
    fout[i] = f;
    a.vx[i] = vx; a.vy[i] = vy; a.vz[i] = vz;
    a.dx[i] += dx; a.dy[i] += dy; a.dz[i] += dz;
    // PASSBOUND is not stored (reference quirk, :372-378)
    if (hi) a.statu[i] = MSMGB_STATU_OUTOFBOX | MSMGB_STATU_REFLECT;
    else if (lo) a.statu[i] = MSMGB_STATU_OUTOFBOX | MSMGB_STATU_TRANSMIT;
    if (hi | lo) atomicOr(&a.flags[kFlagOob], 1);
    // displacement since the last build from the FP32 positions hi + lo (the trigger needs
    // ~1e-4 A, they are within 3e-5 A of the FP64 positions)
    const float4 q = a.pos_bld[i];
    const float4 g = pos_f32(f);
    const float ex = mi32f(g.x - q.x, b.lenf[0], b.halff[0], b.ifpd[0]);
    const float ey = mi32f(g.y - q.y, b.lenf[1], b.halff[1], b.ifpd[1]);
    const float ez = mi32f(g.z - q.z, b.lenf[2], b.halff[2], b.ifpd[2]);
    return ex * ex + ey * ey + ez * ez;
}

// block max of a non-negative float (reduced in FP32, off the FP64 pipe), one atomicMax on
// the bit pattern of its double per block
__device__ __forceinline__ void block_max_flush(float v, unsigned long long *dst)
{
    __shared__ float smf[32];
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(full, v, o));
    if ((threadIdx.x & 31) == 0) smf[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = smf[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, smf[w]);
        // non-negative doubles order like their bit patterns
        if (m > 0.0f) atomicMax(dst, (unsigned long long)__double_as_longlong((double)m));
    }
}

// block max of a non-negative double, one atomicMax (on its bit pattern) per block
__device__ __forceinline__ void block_max_flush(double v, unsigned long long *dst)
{
    __shared__ double sm[32];
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(full, v, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sm[w]);
        // non-negative doubles order like their bit patterns
        if (m > 0.0) atomicMax(dst, (unsigned long long)__double_as_longlong(m));
    }
}

}  // namespace msmgb

struct msmgb_ctx {
    msmgb_params p{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int64_t launches = 0;

    int cap_atoms = 0, cap_boxes = 0;
    int n = 0, nbox = 0;
    std::vector<msmgb_box> boxes;
    std::vector<msmgb::DevBox> hbox;
    int ncell_total = 0, cap_cells = 0;

    // device memory
    msmgb::DevAtoms a{};
    msmgb::DevBox *dbox = nullptr;
    int *cell_of = nullptr, *cell_start = nullptr, *cell_cursor = nullptr, *perm = nullptr;
    int *cell_rank = nullptr;   // storage position of each cell (cells of a box in Morton order)
    int *cell_unrank = nullptr; // global cell id at each storage position
    bool halo_on = false;         // every list build also builds the cell tiles (k_halo)
    // two-level list: candidates within rc_nl + outer_skin, kept between full rebuilds
    double outer_skin = 1.0;      // 0: every rebuild bins, sorts and scans the cell stencil
    double bin_rc = 0.0;          // cell-size radius of the current layout
    double max_density = 0.0;     // atoms per unit volume of the densest box
    int mxo = 0;                  // candidate slots per atom
    int *cand = nullptr;          // candidates, ELL layout [mxo][ld]
    int *kcand = nullptr;         // candidates per atom
    std::vector<double> shapes;   // BOXSHAPE per box (9 each), applied at the next copy-in
    bool any_shaped = false;      // a box of the current state is not cubic
    bool graphs_stale = false;    // a buffer the step graphs hold was reallocated
    bool cell_row_order = false;  // MSMGB_CELL_ORDER=row: x-fastest cell storage instead
    bool check_lists = false;     // MSMGB_CHECK_LISTS=1: validate every list after its build
    std::vector<int> rank_layout; // cell grids (and order) the uploaded cell_rank was made for
    std::vector<double> graph_layout;  // atoms, boxes and cell size the step graphs were captured for
    int *scan_tmp = nullptr;
    void *scratch = nullptr;           // permutation staging (size: 96 B per atom)
    double *cm = nullptr;
    double *icm = nullptr;
    int *flags = nullptr;
    unsigned long long *maxdisp = nullptr;
    double *virial = nullptr;
    int *h_flags = nullptr;            // pinned mirror of flags
    double *h_virial = nullptr;        // pinned

    // tables
    msmgb::DevTables tab{};
    void *tab_mem = nullptr;
    double tab_rmax = 0.0;
    void *adj_mem = nullptr;           // parameter-derivative tables + accumulators
    void *hvp_pair = nullptr;          // HVP: separation, 1/R and SK per list entry (40 B), at first use
    size_t adj_bytes = 0;
    bool have_tables = false;
    bool have_masses = false;

    // external forces added after every force pass (Cumulate_ExtForce0)
    struct ExtForce {
        std::string tag;
        msmgb_extforce_fn fn;
        void *user;
    };
    std::vector<ExtForce> ext;         // registered routines, in order
    double *ext_field = nullptr;       // constant per-atom force, XP(N,3) caller order
    int ext_field_n = 0;               // atom count the field was given for

    bool list_valid = false;
    bool force_valid = false;
    bool den_is32 = false;             // the last density pass was the mixed one

    // autotuned launch variants of the mixed passes (neighbours in flight per thread)
    int tune_dens_unroll = 2, tune_force_unroll = 2, tune_fused = 0;
    float tune_ms_fused = 0.f;
    int tuned_fused_n = -1;      // atom count the fused kernel was tuned for
    // TMA descriptors of the list (INDI) and packed-index (pk) ELL arrays, 2D {ld, mxkvois}
    alignas(64) CUtensorMap tm_indi, tm_pk;
    int tm_state = 0;            // 0 not built, 1 ready, -1 unavailable
    int tuned_n = -1;
    float tune_ms[2] = {0.f, 0.f};

    // second position buffers and graphs of the fused mixed step
    double4_32a *pos2 = nullptr;
    msmgb::PosFF *posff2 = nullptr;
    cudaGraphExec_t g_pre = nullptr, g_loop[2] = {nullptr, nullptr}, g_final[2] = {nullptr, nullptr};
    int64_t gk_pre = 0, gk_loop = 0, gk_final = 0;
    // several steps per graph launch (msmgb_set_steps_per_graph): k step bodies in one graph
    int steps_per_graph = 1;
    cudaGraphExec_t g_loopk[2] = {nullptr, nullptr};   // fused path, first step on buffer p
    cudaGraphExec_t step_graphk = nullptr;             // unfused path
    int64_t gk_loopk = 0, graph_kernels_k = 0;
    int64_t graph_launches = 0;                        // graph launches issued by MD steps
    int64_t gk_body = 0;         // kernels of the conditional rebuild body of a step graph
    int64_t gk_inner = 0;        // two-level list: kernels of the body that runs on every rebuild
    int64_t step_rebuilds = 0, step_full = 0;   // list rebuilds inside MD steps, and the full ones
    double fg_h = 0.0;
    int fg_n = -1, fg_tune = -1, fg_prec = -1;

    // CUDA graph of one MD step
    cudaGraphExec_t step_graph = nullptr;
    int64_t graph_kernels = 0;
    double graph_h = 0.0;
    int graph_prec = -1;
    int graph_n = -1;
    int graph_tune = -1;
};

namespace msmgb {

// --- launch helpers (each increments ctx->launches) -------------------------------------
int check_launch(msmgb_ctx *c, const char *what);
int set_err(msmgb_ctx *c, int code, const std::string &msg);
int cuda_err(msmgb_ctx *c, cudaError_t e, const char *what);

// neighbour list (nlist.cu)
int build_list(msmgb_ctx *c);          // full build (both stages of a two-level list)
bool two_level(const msmgb_ctx *c);     // the list keeps candidates between full rebuilds
int build_full(msmgb_ctx *c);           // binning, sort, permutation, candidates (or the list)
int build_inner(msmgb_ctx *c);          // the list from the candidates (two-level only)
int build_halo(msmgb_ctx *c);
int enable_halo(msmgb_ctx *c);      // allocates the tile buffers, builds them for the current list

// force passes (force64.cu / force32.cu)
int launch_density(msmgb_ctx *c, bool want_epot);
int launch_force(msmgb_ctx *c, bool want_virial);
int launch_stress(msmgb_ctx *c, int sorted, double *ap);
int launch_density32(msmgb_ctx *c);
int launch_force32(msmgb_ctx *c);
int launch_force32_vv(msmgb_ctx *c, double h);
int launch_density_ff(msmgb_ctx *c);
int launch_force_ff(msmgb_ctx *c);
int launch_force_ff_vv(msmgb_ctx *c, double h);
int autotune_fused(msmgb_ctx *c);
int ensure_list_maps(msmgb_ctx *c);
bool uses_tiles(const msmgb_ctx *c);  // a selected mixed variant reads the cell tiles
int launch_wait_selftest(msmgb_ctx *c);
int autotune_mixed(msmgb_ctx *c);
int launch_hvp(msmgb_ctx *c, const double *dv, double *dhv, double *v4buf, double *ddbuf);
int launch_adjoint(msmgb_ctx *c, const double *ft, const double *dtab, double *w4buf, double *ddbuf,
                   double *acc);

// integrator (vv.cu)
int launch_vv(msmgb_ctx *c, double h, int mode);   // mode 0: predictor; 1: fused; 2: fused if pending
int launch_correct(msmgb_ctx *c, double h, bool only_if_pending);
int launch_decide(msmgb_ctx *c, double skin_trigger, int nb_uptab, cudaGraphConditionalHandle cond = 0,
                  bool use_cond = false, cudaGraphConditionalHandle cond_inner = 0);
int launch_set_full(msmgb_ctx *c, cudaGraphConditionalHandle cond_full);

}  // namespace msmgb
