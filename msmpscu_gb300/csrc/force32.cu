// force32.cu -- mixed-precision force passes (FP32 pair, density and table terms).
//
// Same two passes as force64.cu (PRECALFOR_KERNEL / CALFORCE_KERNEL of
// MD_FS_ForceTable_GPU.F90:341-516, 623-806 and the EAM twins), with FP32 arithmetic.
// The reference's tables are linear in sqrt(r) with a step of ~7e-4 A near the first
// neighbour shell, and the Cleri-Rosato exponentials change by ~11x the relative change of r,
// so an index SK = CSI sqrt(r) taken from FP32 r^2 alone would carry ~1e-6 relative error
// into every pair term.  The index is therefore computed from an exact separation:
//   * positions are kept as float-float in the shifted frame u = x - lo + L in [L, 2L], so
//     dh = hi_i - hi_j is exact (Sterbenz) and so is the image shift by float(L); the rest
//     dl = lo_i - lo_j (+ the low part of L) is below 1e-4 A;
//   * r^2 = sum dh^2 + 2 dh dl is formed in float-float (exact squares through fma, exact
//     sums through two-sum); the cutoff test compares it with float-float RU^2, i.e. the
//     FP64 rule up to ~1e-13 relative;
//   * SK = CSI r2^(1/4): two MUFU reciprocal square roots and one Newton correction
//     evaluated in float-float give DK to ~1e-7.
// Hand-over between the passes (one table kind, the common case): the density pass reads one
// 32 B table row {POTB, slope, FPOTR, slope, FPOTB, slope} per pair and hands the force pass
// the interpolated pair terms {FPOTR(r), FPOTB(r)} (8 B per pair, ELL layout; zero beyond RU),
// so the force pass streams them coalesced and gathers no table row; it only forms the FP32
// separation for the force direction and 1/R.  With several table kinds the density pass
// stores the table index of every pair instead (KK << 18 | DK * 2^18, DK quantised to 4e-6,
// a table-value error below 1e-8), because the force pass then needs FPOTB of both KPAIR(i,j)
// and KPAIR(j,i).  Table values come from interleaved {value, slope} FP32 rows; rho and F
// accumulate in FP32 (measured error ~3e-7 of the FP64 forces).  Positions, the integrator
// and the list stay FP64.
#include <algorithm>

#include "msmgb_internal.cuh"

namespace msmgb {

constexpr unsigned kSkip = 0xffffffffu;     // pair beyond RU
constexpr int kDkBits = 18;
constexpr float kDkScale = 262144.0f;       // 2^18
constexpr float kDkInv = 1.0f / 262144.0f;

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

struct BoxF {
    float lh[3], ll[3], half[3];
    int pd[3];
    float dlmax;          // bound on |dl| per component
};

__device__ __forceinline__ BoxF load_boxf(const DevBox &b)
{
    BoxF o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.lh[k] = b.lenf[k];
        o.ll[k] = b.lenlo[k];
        o.half[k] = b.halff[k];
        o.pd[k] = b.ifpd[k];
    }
    o.dlmax = b.dlmax;
    return o;
}

// exact high part and small low part of one separation component (minimum image)
__device__ __forceinline__ void sep2(float hi, float lo, float hj, float lj, float lh, float ll,
                                     float half, int pd, float &dh, float &dl)
{
    dh = hi - hj;                        // exact: both in [L, 2L]
    dl = lo - lj;
    if (pd && fabsf(dh) > half) {
        const float s = copysignf(1.0f, dh);
        dh = fmaf(-s, lh, dh);           // exact (Sterbenz)
        dl = fmaf(-s, ll, dl);
    }
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Packed table index of a pair, or kSkip beyond RU.
__device__ __forceinline__ unsigned pair_index(const PosFF &pi, const PosFF &pj, const BoxF &b,
                                               const DevTables &t, float rej, float &dk_out, int &kk_out)
{
    float xh, xl, yh, yl, zh, zl;
    sep2(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0], xh, xl);
    sep2(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1], yh, yl);
    sep2(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2], zh, zl);
    const float px = xh * xh, py = yh * yh, pz = zh * zh;
    const float approx = px + py + pz;
    // early reject: sum dh^2 differs from r^2 by at most 2 sqrt(3) R max|dl| (+ rounding)
    if (approx > rej) return kSkip;
    float t1, e1, t2, e2;
    two_sum(px, py, t1, e1);
    two_sum(t1, pz, t2, e2);
    const float small = (e1 + e2) + fmaf(xh, xh, -px) + fmaf(yh, yh, -py) + fmaf(zh, zh, -pz) +
                        2.0f * (xh * xl + yh * yl + zh * zl);
    const float r2h = t2 + small;
    const float r2l = small - (r2h - t2);
    if (r2h > t.ru2h || (r2h == t.ru2h && r2l > t.ru2l)) return kSkip;
    // SK = CSI * r2^(1/4), one Newton correction of u = rsqrt(rsqrt(r2)) in float-float
    const float ti = rsqrtf(r2h);
    const float u = rsqrtf(ti);
    const float u2h = u * u, u2l = fmaf(u, u, -u2h);
    const float u4h = u2h * u2h, u4l = fmaf(u2h, u2h, -u4h) + 2.0f * u2h * u2l;
    const float delta = 0.25f * ((r2h - u4h) + (r2l - u4l)) * (ti * ti);
    const float skh = t.csih * u;
    const float skl = fmaf(t.csih, u, -skh) + (t.csih * u) * delta + t.csil * u;
    int kk = (int)skh;
    float dk = (skh - (float)kk) + skl;
    if (dk < 0.0f) { kk -= 1; dk += 1.0f; }
    else if (dk >= 1.0f) { kk += 1; dk -= 1.0f; }
    kk = min(max(kk, 0), t.ntab);
    unsigned q = (unsigned)fminf(fmaf(dk, kDkScale, 0.5f), kDkScale - 1.0f);
    dk_out = dk;
    kk_out = kk;
    return ((unsigned)kk << kDkBits) | q;
}


// combined single-kind table row at index kk: {POTB, dPOTB, FPOTR, dFPOTR}, {FPOTB, dFPOTB, -, -}
__device__ __forceinline__ void ld_comb(const float4 *comb, int kk, float4 &r0, float4 &r1)
{
    const float4 *q = comb + 2 * (size_t)kk;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r0.x), "=f"(r0.y), "=f"(r0.z), "=f"(r0.w), "=f"(r1.x), "=f"(r1.y), "=f"(r1.z), "=f"(r1.w)
        : "l"(q));
}

// One list slot of the density pass.  Single kind: rho contribution and the handed-over pair
// terms {FPOTR(r), FPOTB(r)} (zero beyond RU); several kinds: the packed table index.
template <bool MULTI>
__device__ __forceinline__ float density_slot(const PosFF &pi, const PosFF &pj, const BoxF &b, const DevTables &t,
                                              float rej, int k, bool valid, unsigned *pk, float2 *pb)
{
    float dk = 0.0f;
    int kk = 0;
    const unsigned c = pair_index(pi, pj, b, t, rej, dk, kk);
    const bool ok = valid && c != kSkip;
    if (MULTI) {
        if (valid) *pk = c;
        const float2 e = __ldg(t.dens2 + k * t.ntp + (ok ? kk : 0));
        return ok ? fmaf(dk, e.y, e.x) : 0.0f;
    }
    float4 r0, r1;
    ld_comb(t.comb, ok ? kk : 0, r0, r1);
    if (valid)
        *pb = ok ? make_float2(fmaf(dk, r0.w, r0.z), fmaf(dk, r1.y, r1.x)) : make_float2(0.0f, 0.0f);
    return ok ? fmaf(dk, r0.y, r0.x) : 0.0f;
}

template <int POT, bool MULTI, int UNR, int MINB, bool PF>
__global__ void __launch_bounds__(kBlock, MINB) k_density32(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int kn = a.kvois[i];
    unsigned *__restrict__ pk = a.pk + i;
    float2 *__restrict__ pb = a.pb + i;
    const size_t ld = (size_t)a.ld;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {   // the force pass skips it
        a.den32[i] = 0.0f;
        st_ff(a.rec + i, ld_ff(a.posff + i));          // d = 0
        return;
    }
    const BoxF b = load_boxf(a.box[a.boxid[i]]);
    const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
    const PosFF pi = ld_ff(a.posff + i);
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const int *__restrict__ nb = a.indi + i;
    float rho = 0.0f;
    if (PF) {
        // list entries of the next UNR slots are loaded one iteration ahead (slots past
        // KVOIS are marked -1), so the stream of ELL columns overlaps the position gathers
        int jn[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) jn[u] = u < kn ? __ldg(nb + u * ld) : -1;
        for (int w = 0; w < kn; w += UNR) {
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) j[u] = jn[u];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int sl = w + UNR + u;
                jn[u] = sl < kn ? __ldg(nb + sl * ld) : -1;
            }
            // all gathers first (slots past KVOIS read atom i itself and are discarded)
            PosFF p[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) p[u] = ld_ff(a.posff + (j[u] >= 0 ? j[u] : i));
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int jj = j[u] >= 0 ? j[u] : i;
                const int k = MULTI ? t.kpair[(a.ityp[jj] - 1) * t.ngroup + ti] : 0;
                rho += density_slot<MULTI>(pi, p[u], b, t, rej, k, j[u] >= 0, pk + (w + u) * ld, pb + (w + u) * ld);
            }
        }
    } else {
        int w = 0;
        // UNR neighbours per iteration keep UNR independent gathers in flight
        for (; w + UNR <= kn; w += UNR) {
            int j[UNR];
            PosFF p[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) j[u] = __ldg(nb + (w + u) * ld);
#pragma unroll
            for (int u = 0; u < UNR; ++u) p[u] = ld_ff(a.posff + j[u]);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int k = MULTI ? t.kpair[(a.ityp[j[u]] - 1) * t.ngroup + ti] : 0;
                rho += density_slot<MULTI>(pi, p[u], b, t, rej, k, true, pk + (w + u) * ld, pb + (w + u) * ld);
            }
        }
        for (; w < kn; ++w) {
            const int j0 = __ldg(nb + w * ld);
            const PosFF p0 = ld_ff(a.posff + j0);
            const int k = MULTI ? t.kpair[(a.ityp[j0] - 1) * t.ngroup + ti] : 0;
            rho += density_slot<MULTI>(pi, p0, b, t, rej, k, true, pk + w * ld, pb + w * ld);
        }
    }
    float d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0f) d = -0.5f * rsqrtf(rho);
    } else if (rho > 0.0f) {
        const int ke = MULTI ? t.kembd[ti] : 0;
        const float sk = rho / t.rhodf + 1.0f;
        int kk = (int)(sk + 0.000001f);
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
        }
        const float2 e = __ldg(t.embd2 + ke * t.nep + kk);
        d = fmaf(sk - (float)kk, e.y, e.x);
    }
    a.den32[i] = d;
    PosFF r = pi;
    r.d = d;
    st_ff(a.rec + i, r);
}

// FP32 separation for the force direction (dh exact, dl small)
__device__ __forceinline__ float sep1(float hi, float lo, float hj, float lj, float lh, float ll,
                                      float half, int pd)
{
    float dh, dl;
    sep2(hi, lo, hj, lj, lh, ll, half, pd, dh, dl);
    return dh + dl;
}

// Pair term with several table kinds: table index c from the density pass.
__device__ __forceinline__ void force_pair_multi(const PosFF &pi, const PosFF &pj, unsigned c, float di,
                                                 float dj, int ti, int tj, const BoxF &b, const DevTables &t,
                                                 float &fx, float &fy, float &fz)
{
    const float sx = sep1(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0]);
    const float sy = sep1(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1]);
    const float sz = sep1(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2]);
    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
    const int kk = (int)(c >> kDkBits);
    const float dk = (float)(c & ((1u << kDkBits) - 1)) * kDkInv;
    const int k = t.kpair[tj * t.ngroup + ti];
    const float4 e = __ldg(t.force4 + k * t.ntp + kk);
    const float P = fmaf(dk, e.y, e.x);
    const float B = fmaf(dk, e.w, e.z);
    float emb = B * (di + dj);
    const int k1 = t.kpair[ti * t.ngroup + tj];
    if (k1 != k) {
        const float4 e1 = __ldg(t.force4 + k1 * t.ntp + kk);
        emb = B * di + fmaf(dk, e1.w, e1.z) * dj;
    }
    const float ft = fmaf(P, y, emb) * y;
    fx = fmaf(ft, sx, fx);
    fy = fmaf(ft, sy, fy);
    fz = fmaf(ft, sz, fz);
}

// Pair term with one table kind: the interpolated FPOTR, FPOTB handed over by the density
// pass (both zero beyond RU, so such slots add exactly zero).
__device__ __forceinline__ void force_pair_pb(const PosFF &pi, const PosFF &pj, float2 pbv, float di,
                                              const BoxF &b, float &fx, float &fy, float &fz)
{
    const float sx = sep1(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0]);
    const float sy = sep1(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1]);
    const float sz = sep1(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2]);
    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
    const float ft = fmaf(pbv.x, y, pbv.y * (di + pj.d)) * y;
    fx = fmaf(ft, sx, fx);
    fy = fmaf(ft, sy, fy);
    fz = fmaf(ft, sz, fz);
}

// Walks the ELL list of atom i, UNR slots per iteration, and calls body(j, v) for every slot
// (v = the slot's entry of `pv`, a packed index or handed-over pair terms) for which
// keep(v) holds.  With PF the slots of the next iteration are loaded before the current ones
// are processed (slots past KVOIS read as `none` and are not kept).
template <int UNR, bool PF, class V, class Keep, class Body>
__device__ __forceinline__ void walk_pairs(const int *__restrict__ nb, const V *__restrict__ pv, size_t ld,
                                           int kn, V none, Keep keep, Body body)
{
    if (PF) {
        V cn[UNR];
        int jn[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            cn[u] = u < kn ? __ldg(pv + u * ld) : none;
            jn[u] = u < kn ? __ldg(nb + u * ld) : 0;
        }
        for (int w = 0; w < kn; w += UNR) {
            V c[UNR];
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                c[u] = cn[u];
                j[u] = jn[u];
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int sl = w + UNR + u;
                cn[u] = sl < kn ? __ldg(pv + sl * ld) : none;
                jn[u] = sl < kn ? __ldg(nb + sl * ld) : 0;
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (keep(c[u])) body(j[u], c[u]);
        }
    } else {
        int w = 0;
        for (; w + UNR <= kn; w += UNR) {
            V c[UNR];
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                c[u] = __ldg(pv + (w + u) * ld);
                j[u] = __ldg(nb + (w + u) * ld);
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (keep(c[u])) body(j[u], c[u]);
        }
        for (; w < kn; ++w) {
            const V c0 = __ldg(pv + w * ld);
            if (keep(c0)) body(__ldg(nb + w * ld), c0);
        }
    }
}

struct KeepIndex {
    __device__ bool operator()(unsigned c) const { return c != kSkip; }
};
// slots with zero pair terms (beyond RU, or past KVOIS in the prefetching walk) add nothing
struct KeepTerms {
    __device__ bool operator()(float2 v) const { return v.x != 0.0f || v.y != 0.0f; }
};

// Single-kind force loop with every load of a batch issued before any of its arithmetic: the
// handed-over pair terms and list entries one iteration ahead, then the UNR neighbour records
// {position, F'(rho)} of the batch (slots past KVOIS read atom i itself with zero pair terms).
template <int UNR>
__device__ __forceinline__ void force_loop_batched(const DevAtoms &a, int i, const PosFF &pi, float di,
                                                   const BoxF &b, float &fx, float &fy, float &fz)
{
    const int *__restrict__ nb = a.indi + i;
    const float2 *__restrict__ pb = a.pb + i;
    const size_t ld = (size_t)a.ld;
    const int kn = a.kvois[i];
    const float2 zero = make_float2(0.0f, 0.0f);
    float2 cn[UNR];
    int jn[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
        cn[u] = u < kn ? __ldg(pb + u * ld) : zero;
        jn[u] = u < kn ? __ldg(nb + u * ld) : i;
    }
    for (int w = 0; w < kn; w += UNR) {
        float2 c[UNR];
        int j[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            c[u] = cn[u];
            j[u] = jn[u];
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int sl = w + UNR + u;
            cn[u] = sl < kn ? __ldg(pb + sl * ld) : zero;
            jn[u] = sl < kn ? __ldg(nb + sl * ld) : i;
        }
        PosFF pj[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pj[u] = ld_ff(a.rec + j[u]);
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (j[u] != i) force_pair_pb(pi, pj[u], c[u], di, b, fx, fy, fz);
    }
}

// F_i of one atom of the mixed force pass (PF: 0 plain, 1 list prefetch, 2 prefetch + batched
// gathers; the last only with one table kind)
template <bool MULTI, int UNR, int PF>
__device__ __forceinline__ void force_atom32(const DevAtoms &a, const DevTables &t, int i, float &fx, float &fy,
                                             float &fz)
{
    const BoxF b = load_boxf(a.box[a.boxid[i]]);
    const PosFF pi = ld_ff(a.rec + i);
    const float di = pi.d;
    if (MULTI) {
        const int ti = a.ityp[i] - 1;
        walk_pairs<UNR, (PF != 0)>(a.indi + i, a.pk + i, (size_t)a.ld, a.kvois[i], kSkip, KeepIndex(),
                                   [&](int j, unsigned c) {
                                       const PosFF pj = ld_ff(a.rec + j);
                                       force_pair_multi(pi, pj, c, di, pj.d, ti, a.ityp[j] - 1, b, t, fx, fy, fz);
                                   });
    } else if (PF == 2) {
        force_loop_batched<UNR>(a, i, pi, di, b, fx, fy, fz);
    } else {
        walk_pairs<UNR, (PF != 0)>(a.indi + i, a.pb + i, (size_t)a.ld, a.kvois[i], make_float2(0.0f, 0.0f),
                                   KeepTerms(), [&](int j, float2 v) {
                                       const PosFF pj = ld_ff(a.rec + j);
                                       force_pair_pb(pi, pj, v, di, b, fx, fy, fz);
                                   });
    }
}

template <bool MULTI, int UNR, int MINB, int PF>
__global__ void __launch_bounds__(kBlock, MINB) k_force32(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) force_atom32<MULTI, UNR, PF>(a, t, i, fx, fy, fz);
    a.fx[i] = (double)fx;
    a.fy[i] = (double)fy;
    a.fz[i] = (double)fz;
}

// The mixed MD step kernel (one table kind): force pass, then the corrector of step n and the
// predictor of step n+1 of the same atom (vv_atom), positions of step n+1 into the second
// buffer (neighbours still read step n's records).
template <int UNR, int MINB, int PF>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_vv(DevAtoms a, DevTables t, double th)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dmax = 0.0;
    if (i < a.n) {
        const int stat = a.statu[i];
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;
        const bool act = (stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE;
        if (act) force_atom32<false, UNR, PF>(a, t, i, fx, fy, fz);
        const double Fx = (double)fx, Fy = (double)fy, Fz = (double)fz;
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

// variant codes of the fused kernel: (neighbours in flight, minimum resident blocks), codes
// 6-11 the same six with the next slots of the list loaded one iteration ahead, 12-17 with
// in addition every gather of a batch issued before its arithmetic (force_loop_batched)
constexpr int kFusedVariants = 18;

static void fused_variant(msmgb_ctx *c, int code, double h)
{
    const int g = nblk(c->n, kBlock);
    switch (code) {
    case 1: k_force32_vv<4, 1, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 2: k_force32_vv<2, 4, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 3: k_force32_vv<4, 4, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 4: k_force32_vv<2, 5, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 5: k_force32_vv<4, 5, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 6: k_force32_vv<2, 1, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 7: k_force32_vv<4, 1, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 8: k_force32_vv<2, 4, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 9: k_force32_vv<4, 4, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 10: k_force32_vv<2, 5, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 11: k_force32_vv<4, 5, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 12: k_force32_vv<2, 1, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 13: k_force32_vv<4, 1, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 14: k_force32_vv<2, 4, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 15: k_force32_vv<4, 4, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 16: k_force32_vv<2, 5, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    case 17: k_force32_vv<4, 5, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    default: k_force32_vv<2, 1, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab, h); break;
    }
}

int launch_force32_vv(msmgb_ctx *c, double h)
{
    fused_variant(c, c->tune_fused, h);
    c->launches += 1;
    return check_launch(c, "fused force pass + integrator");
}

// Times the fused variants with h = 0, which leaves positions, velocities and DIS unchanged
// (the next-step buffer receives the current positions), on the atom view c->a.
int autotune_fused(msmgb_ctx *c)
{
    // F'(rho) of the current positions (carried in the float-float records) first, so that
    // the forces the variants write are those of the current state
    int rc = launch_density32(c);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err != cudaSuccess) return cuda_err(c, err, "autotune events");
    float best = 1e30f;
    int bestc = 0;
    for (int code = 0; code < kFusedVariants; ++code) {
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            fused_variant(c, code, 0.0);
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; bestc = code; }
    }
    c->tune_fused = bestc;
    c->tune_ms_fused = best / 3.0f;
    c->tuned_fused_n = c->n;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemsetAsync(c->a.maxdisp, 0, sizeof(unsigned long long), c->stream);
    return check_launch(c, "autotune fused");
}

template <int POT, bool MULTI>
static void dens_variant(msmgb_ctx *c, int unr)
{
    const int g = nblk(c->n, kBlock);
    if (unr & 16) {
        switch (unr & 7) {
        case 4: k_density32<POT, MULTI, 4, 1, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 5: k_density32<POT, MULTI, 4, 6, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 3: k_density32<POT, MULTI, 2, 6, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        default: k_density32<POT, MULTI, 2, 1, true><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        }
        return;
    }
    switch (unr & 7) {
    case 1: k_density32<POT, MULTI, 1, 1, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 4: k_density32<POT, MULTI, 4, 1, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 5: k_density32<POT, MULTI, 4, 6, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 3: k_density32<POT, MULTI, 2, 6, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    default: k_density32<POT, MULTI, 2, 1, false><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    }
}

template <bool MULTI>
static void force_variant(msmgb_ctx *c, int unr)
{
    const int g = nblk(c->n, kBlock);
    if (!MULTI && (unr & 32)) {
        switch (unr & 7) {
        case 4: k_force32<MULTI, 4, 1, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 5: k_force32<MULTI, 4, 6, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 3: k_force32<MULTI, 2, 6, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        default: k_force32<MULTI, 2, 1, 2><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        }
        return;
    }
    if (unr & 16) {
        switch (unr & 7) {
        case 4: k_force32<MULTI, 4, 1, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 5: k_force32<MULTI, 4, 6, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 3: k_force32<MULTI, 2, 6, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        default: k_force32<MULTI, 2, 1, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        }
        return;
    }
    switch (unr & 7) {
    case 1: k_force32<MULTI, 1, 1, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 4: k_force32<MULTI, 4, 1, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 5: k_force32<MULTI, 4, 6, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    case 3: k_force32<MULTI, 2, 6, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    default: k_force32<MULTI, 2, 1, 0><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
    }
}

int launch_density32(msmgb_ctx *c)
{
    if (!c->a.pk || !c->a.pb)
        return set_err(c, MSMGB_ERR_ARG, "mixed passes need the pair buffers (set MIXED precision)");
    if (c->tab.ntab >= (1 << (32 - kDkBits)) - 1)
        return set_err(c, MSMGB_ERR_ARG, "mixed passes support NTAB < 16383");
    const bool multi = c->tab.ngroup > 1;
    const int unr = c->tune_dens_unroll;
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) dens_variant<MSMGB_FS_TYPE, true>(c, unr);
        else dens_variant<MSMGB_FS_TYPE, false>(c, unr);
    } else {
        if (multi) dens_variant<MSMGB_EAM_TYPE, true>(c, unr);
        else dens_variant<MSMGB_EAM_TYPE, false>(c, unr);
    }
    c->launches += 1;
    c->den_is32 = true;
    return check_launch(c, "mixed density pass");
}

int launch_force32(msmgb_ctx *c)
{
    if (c->tab.ngroup > 1) force_variant<true>(c, c->tune_force_unroll);
    else force_variant<false>(c, c->tune_force_unroll);
    c->launches += 1;
    return check_launch(c, "mixed force pass");
}

// Autotuner: times every unroll depth of both mixed passes on the context's current data
// (three launches each after one warm-up, CUDA events on the context stream) and keeps the
// fastest.  Runs once per context and atom count, outside any stream capture.
int autotune_mixed(msmgb_ctx *c)
{
    // code & 7: 1, 2, 4 = neighbours in flight per thread; 3 = 2 and 5 = 4 with registers
    // capped for 6 blocks (75% occupancy); +16: list slots loaded one iteration ahead;
    // +32 (force, single kind): and all gathers of a batch before its arithmetic
    const bool single = c->tab.ngroup == 1;
    const int dcands[9] = {1, 2, 4, 3, 5, 18, 20, 19, 21};
    const int fcands[13] = {1, 2, 4, 3, 5, 18, 20, 19, 21, 50, 52, 51, 53};
    const int *cands = dcands;
    int ncand = 9;
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err != cudaSuccess) return cuda_err(c, err, "autotune events");
    float best_d = 1e30f, best_f = 1e30f;
    int bd = 2, bf = 2;
    for (int k = 0; k < ncand; ++k) {
        c->tune_dens_unroll = cands[k];
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            int rc = launch_density32(c);
            if (rc) return rc;
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_d) { best_d = ms; bd = cands[k]; }
    }
    c->tune_dens_unroll = bd;
    int rc = launch_density32(c);
    if (rc) return rc;
    cands = fcands;
    ncand = single ? 13 : 9;
    for (int k = 0; k < ncand; ++k) {
        c->tune_force_unroll = cands[k];
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            rc = launch_force32(c);
            if (rc) return rc;
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_f) { best_f = ms; bf = cands[k]; }
    }
    c->tune_force_unroll = bf;
    c->tune_ms[0] = best_d / 3.0f;
    c->tune_ms[1] = best_f / 3.0f;
    c->tuned_n = c->n;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return check_launch(c, "autotune");
}

}  // namespace msmgb
