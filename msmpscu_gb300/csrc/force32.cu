// force32.cu -- mixed-precision force passes (FP32 pair, density and table terms).
//
// Same two passes as force64.cu (PRECALFOR_KERNEL / CALFORCE_KERNEL of
// MD_FS_ForceTable_GPU.F90:341-516, 623-806 and the EAM twins), with FP32 arithmetic.
// The reference's tables are linear in sqrt(r) with a step of ~7e-4 A near the first
// neighbour shell, and the Cleri-Rosato exponentials change by ~11x the relative change of r,
// so an index SK = CSI sqrt(r) taken from FP32 r^2 alone would carry ~1e-6 relative error
// into every pair term.  The index is therefore computed from a float-float separation:
//   * positions are kept as float-float in the shifted frame u = x - lo + L in [L, 2L], so
//     hi_i - hi_j is exact (Sterbenz) and so is the image shift by float(L);
//   * r^2 is formed in float-float (exact squares through fma), the cutoff test compares
//     float-float r^2 with float-float RU^2 (the FP64 rule, up to ~1e-13 relative);
//   * SK = CSI r2^(1/4): two MUFU reciprocal square roots and one Newton correction
//     evaluated in float-float, giving DK to ~1e-7.
// Table values come from interleaved {value, slope} FP32 rows (one 8 B or 16 B load per
// pair), accumulation of rho and F is FP32 (measured error ~3e-7 of the FP64 result);
// positions, the integrator and the list stay FP64.
#include "msmgb_internal.cuh"

namespace msmgb {

struct FF {
    float h, l;
};

// exact separation component (hi part exact, lo carries the rest)
__device__ __forceinline__ FF sep_ff(float hi_i, float lo_i, float hi_j, float lo_j, float lh,
                                     float ll, float half, int pd)
{
    float dh = hi_i - hi_j;             // exact: both in [L, 2L]
    float dl = lo_i - lo_j;
    if (pd && fabsf(dh) > half) {
        float s = copysignf(1.0f, dh);
        dh = dh - s * lh;               // exact (Sterbenz)
        dl = dl - s * ll;
    }
    FF r;
    r.h = dh + dl;                      // Fast2Sum: |dh| >= |dl| for all non-coincident atoms
    r.l = dl - (r.h - dh);
    return r;
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

struct PairGeom {
    float sx, sy, sz;     // separation (hi parts)
    float y;              // 1/R
    int kk;               // table index
    float dk;             // fraction in [0, 1)
};

// Returns false when the pair is beyond RU (float-float comparison of r^2 with RU^2).
__device__ __forceinline__ bool pair_geom(const PosFF &pi, const PosFF &pj, const DevBox &b,
                                          const DevTables &t, PairGeom &g)
{
    FF x = sep_ff(pi.hx, pi.lx, pj.hx, pj.lx, b.lenf[0], b.lenlo[0], b.halff[0], b.ifpd[0]);
    FF y = sep_ff(pi.hy, pi.ly, pj.hy, pj.ly, b.lenf[1], b.lenlo[1], b.halff[1], b.ifpd[1]);
    FF z = sep_ff(pi.hz, pi.lz, pj.hz, pj.lz, b.lenf[2], b.lenlo[2], b.halff[2], b.ifpd[2]);
    // float-float r^2
    float px = x.h * x.h, py = y.h * y.h, pz = z.h * z.h;
    float ex = fmaf(x.h, x.h, -px), ey = fmaf(y.h, y.h, -py), ez = fmaf(z.h, z.h, -pz);
    float t1, e1, t2, e2;
    two_sum(px, py, t1, e1);
    two_sum(t1, pz, t2, e2);
    float cross = 2.0f * (x.h * x.l + y.h * y.l + z.h * z.l);
    float lo = (e1 + e2) + (ex + ey + ez) + cross;
    float r2h = t2 + lo;
    float r2l = lo - (r2h - t2);
    if (r2h > t.ru2h || (r2h == t.ru2h && r2l > t.ru2l)) return false;
    // SK = CSI * r2^(1/4) with one Newton correction in float-float
    float ti = rsqrtf(r2h);              // ~ 1/R
    float u = rsqrtf(ti);                // ~ sqrt(R) = r2^(1/4)
    float u2h = u * u, u2l = fmaf(u, u, -u2h);
    float u4h = u2h * u2h, u4l = fmaf(u2h, u2h, -u4h) + 2.0f * u2h * u2l;
    float diff = (r2h - u4h) + (r2l - u4l);
    float delta = 0.25f * diff * (ti * ti);          // relative correction of u
    float skh = t.csih * u;
    float skl = fmaf(t.csih, u, -skh) + t.csih * u * delta + t.csil * u;
    int kk = (int)skh;
    float dk = (skh - (float)kk) + skl;
    if (dk < 0.0f) { kk -= 1; dk += 1.0f; }
    else if (dk >= 1.0f) { kk += 1; dk -= 1.0f; }
    kk = min(max(kk, 0), t.ntab);
    g.sx = x.h; g.sy = y.h; g.sz = z.h;
    g.y = ti;
    g.kk = kk;
    g.dk = dk;
    return true;
}

template <int POT, bool MULTI>
__global__ void __launch_bounds__(kBlock) k_density32(DevAtoms a, DevTables t)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        a.den32[i] = 0.0f;
        return;
    }
    const DevBox &b = a.box[a.boxid[i]];
    const PosFF pi = a.posff[i];
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const int kn = a.kvois[i];
    const int *__restrict__ nb = a.indi + i;
    const size_t ld = (size_t)a.ld;
    float rho = 0.0f;
    for (int w = 0; w < kn; ++w) {
        int j = __ldg(nb + w * ld);
        const PosFF pj = a.posff[j];
        PairGeom g;
        if (!pair_geom(pi, pj, b, t, g)) continue;
        int k = MULTI ? t.kpair[(a.ityp[j] - 1) * t.ngroup + ti] : 0;
        float2 e = __ldg(t.dens2 + (size_t)k * t.ntp + g.kk);
        rho += fmaf(g.dk, e.y, e.x);
    }
    float d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0f) d = -0.5f * rsqrtf(rho);
    } else if (rho > 0.0f) {
        const int ke = MULTI ? t.kembd[ti] : 0;
        float sk = rho / t.rhodf + 1.0f;
        int kk = (int)(sk + 0.000001f);
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
        }
        float2 e = __ldg(t.embd2 + (size_t)ke * t.nep + kk);
        d = fmaf(sk - (float)kk, e.y, e.x);
    }
    a.den32[i] = d;
}

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_force32(DevAtoms a, DevTables t)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &b = a.box[a.boxid[i]];
        const PosFF pi = a.posff[i];
        const int ti = MULTI ? a.ityp[i] - 1 : 0;
        const float di = a.den32[i];
        const int kn = a.kvois[i];
        const int *__restrict__ nb = a.indi + i;
        const size_t ld = (size_t)a.ld;
        for (int w = 0; w < kn; ++w) {
            int j = __ldg(nb + w * ld);
            const PosFF pj = a.posff[j];
            PairGeom g;
            if (!pair_geom(pi, pj, b, t, g)) continue;
            int tj = MULTI ? a.ityp[j] - 1 : 0;
            int k = MULTI ? t.kpair[tj * t.ngroup + ti] : 0;
            float dj = __ldg(a.den32 + j);
            float4 e = __ldg(t.force4 + (size_t)k * t.ntp + g.kk);
            float P = fmaf(g.dk, e.y, e.x);
            float B = fmaf(g.dk, e.w, e.z);
            float B1 = B;
            if (MULTI) {
                int k1 = t.kpair[ti * t.ngroup + tj];
                if (k1 != k) {
                    float4 e1 = __ldg(t.force4 + (size_t)k1 * t.ntp + g.kk);
                    B1 = fmaf(g.dk, e1.w, e1.z);
                }
            }
            float ft = (P * g.y + (B * di + B1 * dj)) * g.y;
            fx = fmaf(ft, g.sx, fx);
            fy = fmaf(ft, g.sy, fy);
            fz = fmaf(ft, g.sz, fz);
        }
    }
    a.fx[i] = (double)fx;
    a.fy[i] = (double)fy;
    a.fz[i] = (double)fz;
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

int launch_density32(msmgb_ctx *c)
{
    int g = nblk(c->n, kBlock);
    bool multi = c->tab.ngroup > 1;
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) k_density32<MSMGB_FS_TYPE, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
        else k_density32<MSMGB_FS_TYPE, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
    } else {
        if (multi) k_density32<MSMGB_EAM_TYPE, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
        else k_density32<MSMGB_EAM_TYPE, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
    }
    c->launches += 1;
    c->den_is32 = true;
    return check_launch(c, "mixed density pass");
}

int launch_force32(msmgb_ctx *c)
{
    int g = nblk(c->n, kBlock);
    if (c->tab.ngroup > 1) k_force32<true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
    else k_force32<false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab);
    c->launches += 1;
    return check_launch(c, "mixed force pass");
}

}  // namespace msmgb
