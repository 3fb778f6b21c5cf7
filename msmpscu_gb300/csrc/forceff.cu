// forceff.cu -- float-float force passes: the FP64 parity form on the FP32 pipe.
//
// Same two passes as force64.cu (PRECALFOR_KERNEL / CALFORCE_KERNEL of
// MD_FS_ForceTable_GPU.F90:341-516, 623-806 and the EAM twins in
// MD_EAM_ForceTable_GPU.F90:369-548, 646-829), evaluated in float-float arithmetic: every
// quantity is an unevaluated sum hi + lo of two FP32 numbers (~48-bit significand).  GB300
// executes FP64 at 1/64 of its FP32 rate, so the FP64 passes are bound by the FP64 pipe;
// these passes meet the same 1e-10 relative parity bar against the FP64 oracle on the FP32
// pipe.  Positions enter as records {hi = float(u), q = (u - hi) / quantum} (k_fix): the hi
// difference is exact (Sterbenz, u in [L, 2L]) and so is the integer difference of the
// remainders, which is converted to float-float only after the subtraction, so a separation
// carries ~3e-14 A (the quantum).  Error budget per pair (relative): separation ~1e-14,
// r^2 and SK ~1e-13 (float-float squares, one Newton step for r2^(1/4) and r2^(-1/2)),
// table values ~1e-14 (tables split into hi + lo, slopes taken in FP64 before the split),
// products and sums 2^-44.
//
//   k_fix         FP64 positions -> position records (once per force evaluation)
//   k_density_ff  rho_i (float-float sum), F'(rho_i) = -1/(2 sqrt(rho)) by a float-float
//                 Newton step (FS) or the DFEMBD interpolant (EAM); writes the record
//                 {position, F'(rho) hi, lo} of atom i for the force pass and F'(rho) as FP64.
//   k_force_ff    recomputes the pair index, 1/R and the FORTOT of every pair in float-float
//                 and accumulates F_i in float-float; writes F as FP64.
//   k_force_ff_vv the same followed by the FP64 corrector / predictor of the atom (the MD step
//                 kernel of this mode, like k_force32_vv of the mixed passes).
#include "msmgb_internal.cuh"

namespace msmgb {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff quick_two_sum(float a, float b)   // |a| >= |b|
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    const ff s = two_sum(x.h, y.h);
    return quick_two_sum(s.h, s.l + (x.l + y.l));
}

__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    const float p = x.h * y.h;
    const float e = fmaf(x.h, y.h, -p);
    return quick_two_sum(p, fmaf(x.h, y.l, fmaf(x.l, y.h, e)));
}

__device__ __forceinline__ ff ff_mul_f(ff x, float f)
{
    const float p = x.h * f;
    const float e = fmaf(x.h, f, -p);
    return quick_two_sum(p, fmaf(x.l, f, e));
}

// Accumulation of a float-float sum without renormalising each term: F.l collects the exact
// rounding errors of the hi additions and the low parts (tiny against F.h), the sum is
// F.h + F.l at the end.
__device__ __forceinline__ void acc_add(ff &F, float ph, float pl)
{
    const ff s = two_sum(F.h, ph);
    F.h = s.h;
    F.l += s.l + pl;
}

// product x*y as an unnormalised pair (p, e) with p + e = x*y to ~2^-46
__device__ __forceinline__ void mul_pair(ff x, ff y, float &p, float &e)
{
    p = x.h * y.h;
    e = fmaf(x.h, y.l, fmaf(x.l, y.h, fmaf(x.h, y.h, -p)));
}

// x + dk * s for a table row {x.h, x.l, s.h, s.l} and dk = dkh + dkl (dkh holds few bits)
__device__ __forceinline__ ff lerp_ff(const float4 &row, float dkh, float dkl)
{
    const ff s = {row.z, row.w};
    const ff d = ff_mul(s, ff{dkh, dkl});
    return ff_add(ff{row.x, row.y}, d);
}

// r^(-1/2) of r = r.h + r.l > 0: FP32 reciprocal square root, one Newton step in float-float
__device__ __forceinline__ ff ff_rsqrt(ff r)
{
    const float y0 = rsqrtf(r.h);
    const ff y2 = {y0 * y0, fmaf(y0, y0, -(y0 * y0))};
    const ff p = ff_mul(r, y2);                       // ~1
    const float e = (1.0f - p.h) - p.l;               // 1 - p.h exact (Sterbenz)
    return quick_two_sum(y0, 0.5f * y0 * e);
}

struct BoxFF {
    float lh[3], half[3];
    int lq[3], pd[3];
    float dlmax, q;
};

__device__ __forceinline__ BoxFF load_boxff(const DevBox &b)
{
    BoxFF o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.lh[k] = b.lenf[k];
        o.half[k] = b.halff[k];
        o.lq[k] = b.lq[k];
        o.pd[k] = b.ifpd[k];
    }
    o.dlmax = b.dlfx;
    o.q = b.fxq;
    return o;
}

// separation component: exact hi difference dh and remainder difference (integer, exact)
// with the minimum image applied to both
__device__ __forceinline__ void sep_fx(float hi, int qi, float hj, int qj, float lh, int lq, float half, int pd,
                                       float &dh, int &dq)
{
    dh = hi - hj;
    dq = qi - qj;
    if (pd && fabsf(dh) > half) {
        const bool pos = dh > 0.0f;
        dh = pos ? dh - lh : dh + lh;                 // exact (Sterbenz)
        dq = pos ? dq - lq : dq + lq;
    }
}

// dh + dq * quantum as float-float (|dq| < 2^31: float(dq) and the integer rest are exact)
__device__ __forceinline__ ff to_ff(float dh, int dq, float quantum)
{
    const float qh = (float)dq;
    const float qr = (float)(dq - (int)qh);
    const ff s = two_sum(dh, qh * quantum);
    return quick_two_sum(s.h, fmaf(qr, quantum, s.l));
}

// Pair geometry: separation, r^2 (float-float), the exact FP64 cut rule, and the table index
// KK with DK = dkh + dkl to ~1e-10.  Returns false beyond RU.
struct PairFF {
    ff s[3];
    ff r2;
    int kk;
    float dkh, dkl;
};

__device__ __forceinline__ bool pair_ff(const PosFX &pi, const PosFX &pj, const BoxFF &b, const DevTables &t,
                                        float rej, PairFF &o)
{
    float dh[3];
    int dq[3];
    sep_fx(pi.hx, pi.qx, pj.hx, pj.qx, b.lh[0], b.lq[0], b.half[0], b.pd[0], dh[0], dq[0]);
    sep_fx(pi.hy, pi.qy, pj.hy, pj.qy, b.lh[1], b.lq[1], b.half[1], b.pd[1], dh[1], dq[1]);
    sep_fx(pi.hz, pi.qz, pj.hz, pj.qz, b.lh[2], b.lq[2], b.half[2], b.pd[2], dh[2], dq[2]);
    // early reject on the hi parts: |remainder difference| <= dlmax per component
    if (dh[0] * dh[0] + dh[1] * dh[1] + dh[2] * dh[2] > rej) return false;
    const ff sx = to_ff(dh[0], dq[0], b.q), sy = to_ff(dh[1], dq[1], b.q), sz = to_ff(dh[2], dq[2], b.q);
    const float xh = sx.h, xl = sx.l, yh = sy.h, yl = sy.l, zh = sz.h, zl = sz.l;
    const float px = xh * xh, py = yh * yh, pz = zh * zh;
    const ff t1 = two_sum(px, py);
    const ff t2 = two_sum(t1.h, pz);
    const float small = (t1.l + t2.l) + fmaf(xh, xh, -px) + fmaf(yh, yh, -py) + fmaf(zh, zh, -pz) +
                        2.0f * (xh * xl + yh * yl + zh * zl);
    const ff r2 = quick_two_sum(t2.h, small);
    if (r2.h > t.ru2h || (r2.h == t.ru2h && r2.l > t.ru2l)) return false;
    // SK = CSI r2^(1/4): u = r2^(1/4) from two reciprocal square roots, one Newton step
    const float ti = rsqrtf(r2.h);
    const float u = rsqrtf(ti);
    const ff u2 = {u * u, fmaf(u, u, -(u * u))};
    const ff u4 = ff_mul(u2, u2);
    const float delta = 0.25f * (((r2.h - u4.h) + (r2.l - u4.l)) * (ti * ti));
    const ff uu = quick_two_sum(u, u * delta);
    const ff sk = ff_mul(ff{t.csih, t.csil}, uu);
    int kk = (int)sk.h;
    float dkh = sk.h - (float)kk;                     // exact
    float dkl = sk.l;
    const float dsum = dkh + dkl;
    if (dsum < 0.0f) { kk -= 1; dkh += 1.0f; }
    else if (dsum >= 1.0f) { kk += 1; dkh -= 1.0f; }
    if (kk < 0) { kk = 0; dkh = 0.0f; dkl = 0.0f; }
    if (kk > t.ntab) { kk = t.ntab; dkh = 0.0f; dkl = 0.0f; }
    o.s[0] = sx;
    o.s[1] = sy;
    o.s[2] = sz;
    o.r2 = r2;
    o.kk = kk;
    o.dkh = dkh;
    o.dkl = dkl;
    return true;
}

__device__ __forceinline__ void st_rec(PosFX *p, const PosFX &r)
{
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(__float_as_int(r.hx)),
                 "r"(__float_as_int(r.hy)), "r"(__float_as_int(r.hz)), "r"(r.qx), "r"(r.qy), "r"(r.qz),
                 "r"(__float_as_int(r.dh)), "r"(__float_as_int(r.dl))
                 : "memory");
}

__device__ __forceinline__ PosFX ld_rec(const PosFX *p)
{
    int v[8];
    asm("ld.global.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p));
    PosFX r;
    r.hx = __int_as_float(v[0]); r.hy = __int_as_float(v[1]); r.hz = __int_as_float(v[2]);
    r.qx = v[3]; r.qy = v[4]; r.qz = v[5];
    r.dh = __int_as_float(v[6]); r.dl = __int_as_float(v[7]);
    return r;
}

// FP64 position -> record (hi, integer remainder); F'(rho) slots zero
__global__ void __launch_bounds__(kBlock) k_fix(DevAtoms a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const DevBox &b = a.box[a.boxid[i]];
    const double4_32a p = a.pos[i];
    const double x[3] = {p.x, p.y, p.z};
    float h[3];
    int q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double u = x[k] + b.ushift[k];
        h[k] = __double2float_rn(u);
        const double r = (u - (double)h[k]) * b.fxinv;          // exact scaling by a power of 2
        q[k] = (int)fmin(fmax(rint(r), -1073741823.0), 1073741823.0);
    }
    PosFX o;
    o.hx = h[0]; o.hy = h[1]; o.hz = h[2];
    o.qx = q[0]; o.qy = q[1]; o.qz = q[2];
    o.dh = 0.0f; o.dl = 0.0f;
    st_rec(a.posfx + i, o);
}

template <int POT, bool MULTI>
__global__ void __launch_bounds__(kBlock) k_density_ff(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const PosFX pi = ld_rec(a.posfx + i);
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        st_rec(a.recfx + i, pi);                      // F'(rho) = 0
        a.den[i] = 0.0;
        return;
    }
    const BoxFF b = load_boxff(a.box[a.boxid[i]]);
    const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const int kn = a.kvois[i];
    const int *__restrict__ nb = a.indi + i;
    const size_t ld = (size_t)a.ld;
    ff rho = {0.0f, 0.0f};
    for (int w = 0; w < kn; ++w) {
        const int j = __ldg(nb + w * ld);
        const PosFX pj = ld_rec(a.posfx + j);
        PairFF q;
        if (!pair_ff(pi, pj, b, t, rej, q)) continue;
        const int k = MULTI ? t.kpair[(a.ityp[j] - 1) * t.ngroup + ti] : 0;
        const float4 row = __ldg(t.densff + (size_t)k * t.ntp + q.kk);
        const ff v = lerp_ff(row, q.dkh, q.dkl);
        acc_add(rho, v.h, v.l);
    }
    rho = quick_two_sum(rho.h, rho.l);
    ff d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho.h > 0.0f) {
            const ff r = ff_rsqrt(rho);
            d = {-0.5f * r.h, -0.5f * r.l};
        }
    } else if (rho.h > 0.0f) {
        // SK = rho / RHOD + 1, KK = int(SK + 1e-6) (MD_EAM_ForceTable_GPU.F90:535-541)
        const int ke = MULTI ? t.kembd[ti] : 0;
        const ff x = ff_mul(rho, ff{t.irhodh, t.irhodl});
        const ff sk = ff_add(x, ff{1.0f, 0.0f});
        int kk = (int)sk.h;
        float fh = sk.h - (float)kk;                  // exact
        const float f = (fh + sk.l) + 0.000001f;
        if (f >= 1.0f) { kk += 1; fh -= 1.0f; }
        else if (f < 0.0f) { kk -= 1; fh += 1.0f; }
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
            const ff rest = ff_add(sk, ff{-(float)kk, 0.0f});
            fh = rest.h;
            d = lerp_ff(__ldg(t.embff + (size_t)ke * t.nep + kk), fh, rest.l);
        } else {
            d = lerp_ff(__ldg(t.embff + (size_t)ke * t.nep + kk), fh, sk.l);
        }
    }
    PosFX r = pi;
    r.dh = d.h;
    r.dl = d.l;
    st_rec(a.recfx + i, r);
    a.den[i] = (double)d.h + (double)d.l;
}

// F_i of one atom in float-float (FORTOT of every pair recomputed from the records)
template <bool MULTI>
__device__ __forceinline__ void force_atom_ff(const DevAtoms &a, const DevTables &t, int i, ff F[3])
{
    const PosFX pi = ld_rec(a.recfx + i);
    const BoxFF b = load_boxff(a.box[a.boxid[i]]);
    const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const ff di = {pi.dh, pi.dl};
    const int kn = a.kvois[i];
    const int *__restrict__ nb = a.indi + i;
    const size_t ld = (size_t)a.ld;
    for (int w = 0; w < kn; ++w) {
        const int j = __ldg(nb + w * ld);
        const PosFX pj = ld_rec(a.recfx + j);
        PairFF q;
        if (!pair_ff(pi, pj, b, t, rej, q)) continue;
        const ff dj = {pj.dh, pj.dl};
        const ff y = ff_rsqrt(q.r2);                              // 1/R
        const float4 *rows = t.forceff;
        int k = 0, k1 = 0;
        if (MULTI) {
            const int tj = a.ityp[j] - 1;
            k = t.kpair[tj * t.ngroup + ti];
            k1 = t.kpair[ti * t.ngroup + tj];
        }
        const float4 *rk = rows + 2 * ((size_t)k * t.ntp + q.kk);
        const ff P = lerp_ff(__ldg(rk), q.dkh, q.dkl);
        const ff B = lerp_ff(__ldg(rk + 1), q.dkh, q.dkl);
        ff emb;
        if (MULTI && k1 != k) {
            const ff B1 = lerp_ff(__ldg(rows + 2 * ((size_t)k1 * t.ntp + q.kk) + 1), q.dkh, q.dkl);
            emb = ff_add(ff_mul(B, di), ff_mul(B1, dj));
        } else {
            emb = ff_mul(B, ff_add(di, dj));
        }
        // FORTOT = (FPOTR / R + (FPOTB_k D_i + FPOTB_k1 D_j)) / R
        const ff ft = ff_mul(ff_add(ff_mul(P, y), emb), y);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float ph, pl;
            mul_pair(ft, q.s[c], ph, pl);
            acc_add(F[c], ph, pl);
        }
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_force_ff(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    ff F[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) force_atom_ff<MULTI>(a, t, i, F);
    a.fx[i] = (double)F[0].h + (double)F[0].l;
    a.fy[i] = (double)F[1].h + (double)F[1].l;
    a.fz[i] = (double)F[2].h + (double)F[2].l;
}

// The float-float MD step kernel: force pass, then corrector of step n and predictor of step
// n+1 of the same atom (vv_atom, FP64), positions of step n+1 into the second buffer.
template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_force_ff_vv(DevAtoms a, DevTables t, double th)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    if (i < a.n) {
        const int stat = a.statu[i];
        ff F[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
        const bool act = (stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE;
        if (act) force_atom_ff<MULTI>(a, t, i, F);
        const double Fx = (double)F[0].h + (double)F[0].l;
        const double Fy = (double)F[1].h + (double)F[1].l;
        const double Fz = (double)F[2].h + (double)F[2].l;
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if (act) {
            dmax = vv_atom(a, i, stat, a.box[a.boxid[i]], th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

int launch_density_ff(msmgb_ctx *c)
{
    if (!c->a.posfx || !c->a.recfx) return set_err(c, MSMGB_ERR_ARG, "float-float passes need their record buffers");
    const int bs = block_for(c->n), g = nblk(c->n, bs);
    k_fix<<<g, bs, 0, c->stream>>>(c->a);
    const bool multi = c->tab.ngroup > 1;
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) k_density_ff<MSMGB_FS_TYPE, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_density_ff<MSMGB_FS_TYPE, false><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    } else {
        if (multi) k_density_ff<MSMGB_EAM_TYPE, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_density_ff<MSMGB_EAM_TYPE, false><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    }
    c->launches += 2;
    c->den_is32 = false;
    return check_launch(c, "float-float density pass");
}

int launch_force_ff_vv(msmgb_ctx *c, double h)
{
    const int g = nblk(c->n, kBlock);
    if (c->tab.ngroup > 1) k_force_ff_vv<true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h);
    else k_force_ff_vv<false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h);
    c->launches += 1;
    return check_launch(c, "float-float force pass + integrator");
}

int launch_force_ff(msmgb_ctx *c)
{
    const int bs = block_for(c->n), g = nblk(c->n, bs);
    if (c->tab.ngroup > 1) k_force_ff<true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    else k_force_ff<false><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    c->launches += 1;
    return check_launch(c, "float-float force pass");
}

}  // namespace msmgb
