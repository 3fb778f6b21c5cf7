// force32.cu -- mixed-precision force passes (FP32 pair, density and table terms).
//
// Same two passes as force64.cu (PRECALFOR_KERNEL / CALFORCE_KERNEL of
// MD_FS_ForceTable_GPU.F90:341-516, 623-806 and the EAM twins), with FP32 arithmetic.
// The reference's tables are linear in sqrt(r) with a step of ~7e-4 A near the first
// neighbour shell, and the Cleri-Rosato exponentials change by ~11x the relative change of r,
// so an index SK = CSI sqrt(r) taken from FP32 r^2 alone would carry ~1e-6 relative error
// into every pair term.  The index is therefore computed from an exact separation:
//   * positions are kept as float-float in the shifted frame u = x - lo + L in [L, 2L], the
//     hi parts on a power-of-two quantum, so dh = hi_i - hi_j is exact and so is the image
//     shift by L rounded to the quantum; the rest dl = lo_i - lo_j (+ the rest of L) is below
//     the quantum;
//   * r^2 = sum dh^2 + sum dl (2 dh + dl) as a float-float pair (sum dh^2 exact in FP32); the
//     cutoff test compares it with float-float RU^2;
//   * SK from one table row holding r2_k = (k/CSI)^4 (k_density32q) or from two MUFU
//     reciprocal square roots and one Newton correction in float-float (k_density32).
// The density pass stores the table index of every pair it accepts (KK << 18 | DK * 2^18,
// DK quantised to 4e-6, i.e. a table-value error below 1e-8) in the ELL layout of the
// list; the force pass reads it back instead of recomputing the separation in float-float
// and only forms an FP32 separation for the force direction and 1/R.
// Table values come from interleaved {value, slope} FP32 rows (one 8 B or 16 B load per
// pair); rho and F accumulate in compensated FP32 (measured error ~3e-7 of the FP64 forces).
// Positions, the integrator and the list stay FP64.  The density pass also writes each
// atom's {position, F'(rho)} record, 32 B float-float and, while every box edge span is
// within 1,024 A, 16 B fixed-point (coordinates as 32-bit fractions of the box), so the force
// pass gets both with one gather; on the fixed-point records a separation is the wrapping
// int32 difference times the unit.
// Every pass exists in several variants (neighbours in flight, register caps, list
// prefetch, batched gathers, one-box constants, the two record formats, TMA-streamed list
// tiles, cell tiles, shared-memory table windows) that the autotuner times once per atom
// count.
#include <algorithm>
#include <cstring>
#include <cstdio>
#include <cstdlib>

#include <vector>

#include "msmgb_internal.cuh"

namespace msmgb {

constexpr unsigned kSkip = 0xffffffffu;     // pair beyond RU

// The density pass's per-atom output: the 32 B float-float record {position, F'(rho)} and,
// when the fixed-point records are on, the 16 B record the fixed-point force variants gather.
__device__ __forceinline__ void store_rec(const DevAtoms &a, int i, const PosFF &r)
{
    st_ff(a.rec + i, r);
    if (a.fix_on) a.rec16[i] = fix_record(r, r.d, a.box[a.boxid[i]]);
}

// MSMGB_TUNE_LOG=1: the autotuners print every variant's time per launch to stderr
static bool tune_log()
{
    const char *v = getenv("MSMGB_TUNE_LOG");
    return v && v[0] == '1';
}
constexpr int kDkBits = 18;
constexpr float kDkScale = 262144.0f;       // 2^18
constexpr float kDkInv = 1.0f / 262144.0f;

// Compensated (Kahan) FP32 sum of the pair terms: s - c carries the sum of the rounded terms
// to about twice FP32 precision, so the order and number of the ~46 terms do not add to the
// error of a density or force component.
struct KSum {
    float s = 0.0f, c = 0.0f;       // running sum, its lost low part (negated)
    __device__ __forceinline__ void add(float x)
    {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ void fma_add(float a, float b)     // += a * b
    {
        const float y = fmaf(a, b, -c);
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
    __device__ __forceinline__ double value64() const { return (double)s - (double)c; }
};

struct BoxF {
    float lh[3], ll[3], half[3];
    int pd[3];
    float dlmax;          // bound on |dl| per component
};

__host__ __device__ __forceinline__ BoxF load_boxf(const DevBox &b)
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
    // the lo parts (up to the positions' quantum) enter as dl (2 dh + dl)
    const float small = (e1 + e2) + fmaf(xh, xh, -px) + fmaf(yh, yh, -py) + fmaf(zh, zh, -pz) +
                        (xl * fmaf(2.0f, xh, xl) + yl * fmaf(2.0f, yh, yl) + zl * fmaf(2.0f, zh, zl));
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

template <int POT, bool MULTI, int UNR, int MINB, bool PF>
__global__ void __launch_bounds__(kBlock, MINB) k_density32(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int kn = a.kvois[i];
    unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {   // the force pass skips it
        a.den32[i] = 0.0f;
        store_rec(a, i, ld_ff(a.posff + i));          // d = 0
        return;
    }
    const BoxF b = load_boxf(a.box[a.boxid[i]]);
    const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
    const PosFF pi = ld_ff(a.posff + i);
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const int *__restrict__ nb = a.indi + i;
    const float2 *__restrict__ row0 = t.dens2;
    KSum racc;
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
                float dk = 0.0f;
                int kk = 0;
                const unsigned c = pair_index(pi, p[u], b, t, rej, dk, kk);
                if (j[u] >= 0) pk[(w + u) * ld] = c;
                const bool ok = j[u] >= 0 && c != kSkip;
                const int k = MULTI ? t.kpair[(a.ityp[j[u] >= 0 ? j[u] : i] - 1) * t.ngroup + ti] : 0;
                const float2 e = __ldg(row0 + k * t.ntp + (ok ? kk : 0));
                if (ok) racc.add(fmaf(dk, e.y, e.x));   // a skipped slot adds nothing (not even 0)
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
                float dk;
                int kk;
                const unsigned c = pair_index(pi, p[u], b, t, rej, dk, kk);
                pk[(w + u) * ld] = c;
                if (c != kSkip) {
                    const int k = MULTI ? t.kpair[(a.ityp[j[u]] - 1) * t.ngroup + ti] : 0;
                    const float2 e = __ldg(row0 + k * t.ntp + kk);
                    racc.add(fmaf(dk, e.y, e.x));
                }
            }
        }
        for (; w < kn; ++w) {
            const int j0 = __ldg(nb + w * ld);
            const PosFF p0 = ld_ff(a.posff + j0);
            float dk;
            int kk;
            const unsigned c = pair_index(pi, p0, b, t, rej, dk, kk);
            pk[w * ld] = c;
            if (c != kSkip) {
                const int k = MULTI ? t.kpair[(a.ityp[j0] - 1) * t.ngroup + ti] : 0;
                const float2 e = __ldg(row0 + k * t.ntp + kk);
                racc.add(fmaf(dk, e.y, e.x));
            }
        }
    }
    const float rho = racc.value();
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
    store_rec(a, i, r);
}

// ---- table-assisted density pass --------------------------------------------------------
// The same pass as k_density32 (same pk codes, rho within FP32 rounding of the terms) with
// fewer instructions per pair:
//   * exact sum of squares: the hi parts of the positions are multiples of the box quantum q,
//     a power of two with every component of an accepted pair below 2^11 q (RU below ~18 A at
//     the smallest q, 2^-7 A); the hi differences dh are exact multiples of q and
//     dhx^2 + dhy^2 + dhz^2 is an integer times q^2 below 2^24 q^2, exact in FP32; the lo
//     parts' difference dl (below q) enters r^2 as C = sum dl (2 dh + dl), and the cutoff test
//     and D below take S and C as they are (S - RU^2 and S - r2_k exact by Sterbenz);
//   * the sqrt(r) index by one table row: SK0 = CSI rsqrt(rsqrt(r^2)) (FP32) gives the grid
//     point k = int(SK0); the row holds r2_k = (k/CSI)^4 as float-float, and with
//     D = r^2 - r2_k (exact difference) the fraction is
//         DK = SK - k = (SK/(4 r^2)) D (1 + 3/8 D/r^2)  (Taylor expansion of SK(r^2) about r^2,
//     third-order rest below 1e-6 of DK for k >= 1000, i.e. r > (1000/CSI)^2), instead of a
//     Newton correction in float-float; the same row carries POTB(k) and its slope.
// When FP32 rounding puts SK0 in the neighbouring segment, DK lands just outside [0, 1): the
// pk code is then moved to the reference's segment (k -/+ 1), and rho takes the value of
// segment k extended by at most 2e-3 of a step (a difference below 1e-8 of the term).
struct QBox {
    float lq[3], ll[3], half[3];    // box edge rounded to a multiple of q, and its rest
    int pd;                         // periodic directions, bit k
};

__host__ __device__ __forceinline__ float qround(float h, float m)   // nearest multiple of q (m = 1.5 2^23 q)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(__fadd_rn(h, m), m);
#else
    volatile float s = h + m;            // IEEE single additions on the host as on the device
    return s - m;
#endif
}

__host__ __device__ __forceinline__ QBox qbox_of(const DevBox &bb, float qm)
{
    QBox b;
    for (int k = 0; k < 3; ++k) {
        b.lq[k] = qround(bb.lenf[k], qm);
#ifdef __CUDA_ARCH__
        b.ll[k] = __fadd_rn(__fsub_rn(bb.lenf[k], b.lq[k]), bb.lenlo[k]);
#else
        volatile float d = bb.lenf[k] - b.lq[k];
        b.ll[k] = d + bb.lenlo[k];
#endif
        b.half[k] = bb.halff[k];
    }
    b.pd = (bb.ifpd[0] ? 1 : 0) | (bb.ifpd[1] ? 2 : 0) | (bb.ifpd[2] ? 4 : 0);
    return b;
}

// SB (one box): the box constants come from the kernel parameter qbp (the constant bank)
// instead of per-thread registers loaded from the box array.  PER: every box is periodic along
// all three edges (no per-edge periodicity test in the image).
template <int POT, int UNR, int MINB, bool PF, bool SB = false, bool PER = false>
__global__ void __launch_bounds__(kBlock, MINB) k_density32q(DevAtoms a, DevTables t, float qm, float rejs,
                                                             QBox qbp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int kn = a.kvois[i];
    unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        a.den32[i] = 0.0f;
        store_rec(a, i, ld_ff(a.posff + i));
        return;
    }
    QBox bl;
    if (!SB) {
        const DevBox &bb = a.box[a.boxid[i]];
        bl = qbox_of(bb, qm);
    }
    const QBox &b = SB ? qbp : bl;
    const PosFF pi = ld_ff(a.posff + i);
    const float ih[3] = {pi.hx, pi.hy, pi.hz}, il[3] = {pi.lx, pi.ly, pi.lz};
    const int *__restrict__ nb = a.indi + i;
    const float4 *__restrict__ rows = t.densq;
    KSum racc;
    auto pair = [&](const PosFF &pj, unsigned &code) -> float {
        const float h[3] = {pj.hx, pj.hy, pj.hz}, l[3] = {pj.lx, pj.ly, pj.lz};
        float dh[3], dl[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dh[k] = ih[k] - h[k];                                 // exact multiple of q
            dl[k] = il[k] - l[k];
            if ((PER || ((b.pd >> k) & 1)) && fabsf(dh[k]) > b.half[k]) {
                const float sg = copysignf(1.0f, dh[k]);
                dh[k] = fmaf(-sg, b.lq[k], dh[k]);                // exact
                dl[k] = fmaf(-sg, b.ll[k], dl[k]);
            }
        }
        const float S = fmaf(dh[0], dh[0], fmaf(dh[1], dh[1], dh[2] * dh[2]));   // exact
        code = kSkip;
        if (S > rejs) return 0.0f;
        const float C = fmaf(dl[0], fmaf(2.0f, dh[0], dl[0]),
                             fmaf(dl[1], fmaf(2.0f, dh[1], dl[1]), dl[2] * fmaf(2.0f, dh[2], dl[2])));
        // the cutoff rule r^2 = S + C <= RU^2 and D = r^2 - r2_k without forming r^2 as a
        // float-float pair: S - RU^2_hi and S - r2_k hi are exact (Sterbenz) where it matters
        if ((S - t.ru2h) + (C - t.ru2l) > 0.0f) return 0.0f;
        const float ti = rsqrtf(S + C);
        const float sk0 = t.csih * rsqrtf(ti);          // >= 0
        int kk = min((int)sk0, t.ntab);
        const float4 e = __ldg(rows + kk);
        const float d = (S - e.z) + (C - e.w);
        const float x = d * (ti * ti);
        float dk = 0.25f * sk0 * x * fmaf(0.375f, x, 1.0f);
        const float v = fmaf(dk, e.y, e.x);
        // DK just outside [0, 1) moves the code to the neighbouring segment (dk - floor(dk) is
        // exact)
        const float fl = floorf(dk);
        kk = min(max(kk + (int)fl, 0), t.ntab);
        dk -= fl;
        const unsigned q = (unsigned)fminf(fmaf(dk, kDkScale, 0.5f), kDkScale - 1.0f);
        code = ((unsigned)kk << kDkBits) | q;
        return v;
    };
    if (PF) {
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
            PosFF p[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) p[u] = ld_ff(a.posff + (j[u] >= 0 ? j[u] : i));
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                unsigned c;
                const float v = pair(p[u], c);
                if (j[u] >= 0) {
                    pk[(w + u) * ld] = c;
                    if (c != kSkip) racc.add(v);
                }
            }
        }
    } else {
        int w = 0;
        for (; w + UNR <= kn; w += UNR) {
            int j[UNR];
            PosFF p[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) j[u] = __ldg(nb + (w + u) * ld);
#pragma unroll
            for (int u = 0; u < UNR; ++u) p[u] = ld_ff(a.posff + j[u]);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                unsigned c;
                const float v = pair(p[u], c);
                pk[(w + u) * ld] = c;
                if (c != kSkip) racc.add(v);
            }
        }
        for (; w < kn; ++w) {
            unsigned c;
            const float v = pair(ld_ff(a.posff + __ldg(nb + w * ld)), c);
            pk[w * ld] = c;
            if (c != kSkip) racc.add(v);
        }
    }
    const float rho = racc.value();
    float d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0f) d = -0.5f * rsqrtf(rho);
    } else if (rho > 0.0f) {
        const float sk = rho / t.rhodf + 1.0f;
        int kk = (int)(sk + 0.000001f);
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
        }
        const float2 e = __ldg(t.embd2 + kk);
        d = fmaf(sk - (float)kk, e.y, e.x);
    }
    a.den32[i] = d;
    PosFF r = pi;
    r.d = d;
    store_rec(a, i, r);
}

// Constants of the table-assisted density pass for the current tables and boxes, false when
// the pass does not apply: the positions' quantum q (the same for every box) must satisfy
// 3 (RU + 0.05)^2 < (2^12 q)^2, so that the sum of squares of the hi differences of an
// accepted pair (components below RU + 1.5 q) is exact.  qm = 1.5 2^23 q rounds the box edges
// to q; rejs bounds S of an accepted pair: r^2 - S = C, |C| <= 3 sqrt(3) RU q + 7 q^2
// (|dl| <= 1.5 q).
static bool density_q_params(const msmgb_ctx *c, float *qm, float *rejs)
{
    if (c->hbox.empty()) return false;
    const double ru = std::sqrt(c->tab.ru2);
    const double q = c->hbox[0].qq;
    if ((ru + 0.05) * std::sqrt(3.0) / 4096.0 > q) return false;
    *qm = c->hbox[0].qmag;
    *rejs = (float)(c->tab.ru2 * (1.0 + 1e-5) + 3.0 * std::sqrt(3.0) * ru * q + 7.0 * q * q);
    return true;
}

// FP32 separation for the force direction (dh exact, dl small)
__device__ __forceinline__ float sep1(float hi, float lo, float hj, float lj, float lh, float ll,
                                      float half, int pd)
{
    float dh, dl;
    sep2(hi, lo, hj, lj, lh, ll, half, pd, dh, dl);
    return dh + dl;
}

template <bool MULTI>
__device__ __forceinline__ void force_pair(const PosFF &pi, const PosFF &pj, unsigned c, float di,
                                           float dj, int ti, int tj, const BoxF &b, const DevTables &t,
                                           KSum &fx, KSum &fy, KSum &fz)
{
    const float sx = sep1(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0]);
    const float sy = sep1(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1]);
    const float sz = sep1(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2]);
    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
    const int kk = (int)(c >> kDkBits);
    const float dk = (float)(c & ((1u << kDkBits) - 1)) * kDkInv;
    const int k = MULTI ? t.kpair[tj * t.ngroup + ti] : 0;
    const float4 e = __ldg(t.force4 + k * t.ntp + kk);
    const float P = fmaf(dk, e.y, e.x);
    const float B = fmaf(dk, e.w, e.z);
    float emb = B * (di + dj);
    if (MULTI) {
        const int k1 = t.kpair[ti * t.ngroup + tj];
        if (k1 != k) {
            const float4 e1 = __ldg(t.force4 + k1 * t.ntp + kk);
            emb = B * di + fmaf(dk, e1.w, e1.z) * dj;
        }
    }
    const float ft = fmaf(P, y, emb) * y;
    fx.fma_add(ft, sx);
    fy.fma_add(ft, sy);
    fz.fma_add(ft, sz);
}

// Walks the ELL list of atom i, UNR slots per iteration, and calls body(j, c) for every slot
// whose packed index c is not kSkip.  With PF the slots of the next iteration are loaded
// before the current ones are processed (slots past KVOIS read as kSkip).
template <int UNR, bool PF, class Body>
__device__ __forceinline__ void walk_pairs(const int *__restrict__ nb, const unsigned *__restrict__ pk,
                                           size_t ld, int kn, Body body)
{
    if (PF) {
        unsigned cn[UNR];
        int jn[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            cn[u] = u < kn ? __ldg(pk + u * ld) : kSkip;
            jn[u] = u < kn ? __ldg(nb + u * ld) : 0;
        }
        for (int w = 0; w < kn; w += UNR) {
            unsigned c[UNR];
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                c[u] = cn[u];
                j[u] = jn[u];
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int sl = w + UNR + u;
                cn[u] = sl < kn ? __ldg(pk + sl * ld) : kSkip;
                jn[u] = sl < kn ? __ldg(nb + sl * ld) : 0;
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (c[u] != kSkip) body(j[u], c[u]);
        }
    } else {
        int w = 0;
        for (; w + UNR <= kn; w += UNR) {
            unsigned c[UNR];
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                c[u] = __ldg(pk + (w + u) * ld);
                j[u] = __ldg(nb + (w + u) * ld);
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (c[u] != kSkip) body(j[u], c[u]);
        }
        for (; w < kn; ++w) {
            const unsigned c0 = __ldg(pk + w * ld);
            if (c0 != kSkip) body(__ldg(nb + w * ld), c0);
        }
    }
}

// Single-kind pair term with the table row e = {P, P', B, B'} (at KK) already loaded.
__device__ __forceinline__ void force_pair_e(const PosFF &pi, const PosFF &pj, unsigned c, float di, float dj,
                                             const float4 &e, const BoxF &b, KSum &fx, KSum &fy, KSum &fz)
{
    const float sx = sep1(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0]);
    const float sy = sep1(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1]);
    const float sz = sep1(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2]);
    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
    const float dk = (float)(c & ((1u << kDkBits) - 1)) * kDkInv;
    const float P = fmaf(dk, e.y, e.x);
    const float B = fmaf(dk, e.w, e.z);
    const float ft = fmaf(P, y, B * (di + dj)) * y;
    fx.fma_add(ft, sx);
    fy.fma_add(ft, sy);
    fz.fma_add(ft, sz);
}

// Single-kind force loop over the ELL list of atom i with every load of a batch issued
// before any of its arithmetic: list slots one iteration ahead, then for all UNR slots the
// neighbour position with its F'(rho) (one 32 B record) and the table row.  Slots beyond RU (kSkip) and past
// KVOIS gather row 0 / atom i itself, which are always valid addresses, and are then not
// accumulated.  The loads are thereby unconditional and overlap, instead of one dependent
// gather chain per slot.
template <int UNR>
__device__ __forceinline__ void force_loop_batched(const DevAtoms &a, const DevTables &t, int i, const PosFF &pi,
                                                   float di, const BoxF &b, KSum &fx, KSum &fy, KSum &fz)
{
    const int *__restrict__ nb = a.indi + i;
    const unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    const int kn = a.kvois[i];
    unsigned cn[UNR];
    int jn[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
        cn[u] = u < kn ? __ldg(pk + u * ld) : kSkip;
        jn[u] = u < kn ? __ldg(nb + u * ld) : i;
    }
    for (int w = 0; w < kn; w += UNR) {
        unsigned c[UNR];
        int j[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            c[u] = cn[u];
            j[u] = jn[u];
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int sl = w + UNR + u;
            cn[u] = sl < kn ? __ldg(pk + sl * ld) : kSkip;
            jn[u] = sl < kn ? __ldg(nb + sl * ld) : i;
        }
        PosFF pj[UNR];
        float4 e[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const unsigned row = c[u] == kSkip ? 0u : (c[u] >> kDkBits);
            pj[u] = ld_ff(a.rec + j[u]);
            e[u] = __ldg(t.force4 + row);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (c[u] != kSkip) force_pair_e(pi, pj[u], c[u], di, pj[u].d, e[u], b, fx, fy, fz);
    }
}

// ---- fixed-point records ----------------------------------------------------------------
// The force loop below gathers each neighbour's 16 B fixed-point record (fix_record) instead of
// its 32 B float-float one: a separation component is (float)(int)(q_i - q_j) * unit, the
// wrapping int32 difference being the minimum image along a periodic edge, so the image test
// and the lo parts disappear from the pair term and a lane's gather is half a sector.  The
// table index is still the density pass's exact one (pk); only the direction and 1/R come
// from the fixed-point separation (~1e-7 of its length against ~6e-8 for the float-float one).

// The pair term on two fixed-point records as the three products ft s_k (zero for a skipped
// slot)
__device__ __forceinline__ void pair_terms_fix(const uint4 &pi, const uint4 &pj, unsigned c, float di,
                                               const float4 &e, const float *fu, float &tx, float &ty,
                                               float &tz)
{
    const float sx = (float)(int)(pi.x - pj.x) * fu[0];
    const float sy = (float)(int)(pi.y - pj.y) * fu[1];
    const float sz = (float)(int)(pi.z - pj.z) * fu[2];
    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
    const float dk = (float)(c & ((1u << kDkBits) - 1)) * kDkInv;
    const float P = fmaf(dk, e.y, e.x);
    const float B = fmaf(dk, e.w, e.z);
    const float ft = c != kSkip ? fmaf(P, y, B * (di + __uint_as_float(pj.w))) * y : 0.0f;
    tx = ft * sx;
    ty = ft * sy;
    tz = ft * sz;
}

// force_loop_batched on the fixed-point records (pi: atom i's record, fu: its box's units).
// The pair terms of list slots 2m and 2m + 1 are added in FP32 and their sum enters the
// compensated sum, so its four additions per component are paid once per two slots; the
// pairing follows the slots, not the batch (UNR is even), so every variant sums alike.
template <int UNR>
__device__ __forceinline__ void force_loop_fix(const DevAtoms &a, const DevTables &t, int i, const uint4 &pi,
                                               const float *fu, KSum &fx, KSum &fy, KSum &fz)
{
    const int *__restrict__ nb = a.indi + i;
    const unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    const int kn = a.kvois[i];
    const float di = __uint_as_float(pi.w);
    unsigned cn[UNR];
    int jn[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
        cn[u] = u < kn ? __ldg(pk + u * ld) : kSkip;
        jn[u] = u < kn ? __ldg(nb + u * ld) : i;
    }
    for (int w = 0; w < kn; w += UNR) {
        unsigned c[UNR];
        int j[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            c[u] = cn[u];
            j[u] = jn[u];
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int sl = w + UNR + u;
            cn[u] = sl < kn ? __ldg(pk + sl * ld) : kSkip;
            jn[u] = sl < kn ? __ldg(nb + sl * ld) : i;
        }
        uint4 pj[UNR];
        float4 e[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const unsigned row = c[u] == kSkip ? 0u : (c[u] >> kDkBits);
            pj[u] = __ldg(a.rec16 + j[u]);
            e[u] = __ldg(t.force4 + row);
        }
        static_assert(UNR % 2 == 0, "slots are paired");
        float tx[UNR], ty[UNR], tz[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pair_terms_fix(pi, pj[u], c[u], di, e[u], fu, tx[u], ty[u], tz[u]);
#pragma unroll
        for (int u = 0; u < UNR; u += 2) {
            fx.add(tx[u] + tx[u + 1]);
            fy.add(ty[u] + ty[u + 1]);
            fz.add(tz[u] + tz[u + 1]);
        }
    }
}

// the mixed force pass (single kind) on the fixed-point records
template <int UNR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_fix(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    KSum fx, fy, fz;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &bb = a.box[a.boxid[i]];
        const float fu[3] = {bb.fixu[0], bb.fixu[1], bb.fixu[2]};
        force_loop_fix<UNR>(a, t, i, __ldg(a.rec16 + i), fu, fx, fy, fz);
    }
    // the compensated sums finished in FP32 as in the fused kernel on these records
    a.fx[i] = (double)fx.value();
    a.fy[i] = (double)fy.value();
    a.fz[i] = (double)fz.value();
}

template <bool MULTI, int UNR, int MINB, int PF>
__global__ void __launch_bounds__(kBlock, MINB) k_force32(DevAtoms a, DevTables t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    KSum fx, fy, fz;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const BoxF b = load_boxf(a.box[a.boxid[i]]);
        const PosFF pi = ld_ff(a.rec + i);
        const int ti = MULTI ? a.ityp[i] - 1 : 0;
        const float di = pi.d;
        if (PF == 2 && !MULTI) {
            force_loop_batched<UNR>(a, t, i, pi, di, b, fx, fy, fz);
        } else {
            walk_pairs<UNR, (PF != 0)>(a.indi + i, a.pk + i, (size_t)a.ld, a.kvois[i], [&](int j, unsigned c) {
                const PosFF pj = ld_ff(a.rec + j);
                force_pair<MULTI>(pi, pj, c, di, pj.d, ti, MULTI ? a.ityp[j] - 1 : 0, b, t, fx, fy, fz);
            });
        }
    }
    a.fx[i] = fx.value64();
    a.fy[i] = fy.value64();
    a.fz[i] = fz.value64();
}

// ---- persistent variants with the used table range in shared memory -----------------
// One block per SM slot (grid = resident blocks x SMs), grid-stride over the atoms.  The
// last `cnt` rows of the single-kind table (the short-distance end is rarely reached) are
// copied to shared memory once per block, so the divergent per-lane table reads of a warp
// hit shared memory banks instead of distinct L1 lines; rows below `kmin` fall back to the
// global table.
template <int POT, int UNR>
__global__ void __launch_bounds__(kBlock) k_density32s(DevAtoms a, DevTables t, int kmin, int cnt)
{
    extern __shared__ float2 sdens[];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) sdens[k] = t.dens2[kmin + k];
    __syncthreads();
    const size_t ld = (size_t)a.ld;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const int kn = a.kvois[i];
        unsigned *__restrict__ pk = a.pk + i;
        if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
            a.den32[i] = 0.0f;
            store_rec(a, i, ld_ff(a.posff + i));
            continue;
        }
        const BoxF b = load_boxf(a.box[a.boxid[i]]);
        const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
        const PosFF pi = ld_ff(a.posff + i);
        const int *__restrict__ nb = a.indi + i;
        KSum racc;
        int w = 0;
        for (; w + UNR <= kn; w += UNR) {
            int j[UNR];
            PosFF p[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) j[u] = __ldg(nb + (w + u) * ld);
#pragma unroll
            for (int u = 0; u < UNR; ++u) p[u] = ld_ff(a.posff + j[u]);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                float dk;
                int kk;
                const unsigned c = pair_index(pi, p[u], b, t, rej, dk, kk);
                pk[(w + u) * ld] = c;
                if (c != kSkip) {
                    const float2 e = kk >= kmin ? sdens[kk - kmin] : __ldg(t.dens2 + kk);
                    racc.add(fmaf(dk, e.y, e.x));
                }
            }
        }
        for (; w < kn; ++w) {
            const int j0 = __ldg(nb + w * ld);
            const PosFF p0 = ld_ff(a.posff + j0);
            float dk;
            int kk;
            const unsigned c = pair_index(pi, p0, b, t, rej, dk, kk);
            pk[w * ld] = c;
            if (c != kSkip) {
                const float2 e = kk >= kmin ? sdens[kk - kmin] : __ldg(t.dens2 + kk);
                racc.add(fmaf(dk, e.y, e.x));
            }
        }
        const float rho = racc.value();
        float d = rho;
        if (POT == MSMGB_FS_TYPE) {
            if (rho > 0.0f) d = -0.5f * rsqrtf(rho);
        } else if (rho > 0.0f) {
            const float sk = rho / t.rhodf + 1.0f;
            int kk = (int)(sk + 0.000001f);
            if (kk + 1 > t.nembd) {
                atomicOr(&a.flags[kFlagErr], kErrRho);
                kk = t.nembd;
            }
            const float2 e = __ldg(t.embd2 + kk);
            d = fmaf(sk - (float)kk, e.y, e.x);
        }
        a.den32[i] = d;
        PosFF r = pi;
        r.d = d;
        store_rec(a, i, r);
    }
}

template <int UNR>
__global__ void __launch_bounds__(kBlock) k_force32s(DevAtoms a, DevTables t, int kmin, int cnt)
{
    extern __shared__ float4 sforce[];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) sforce[k] = t.force4[kmin + k];
    __syncthreads();
    const size_t ld = (size_t)a.ld;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        KSum fx, fy, fz;
        if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const BoxF b = load_boxf(a.box[a.boxid[i]]);
            const PosFF pi = ld_ff(a.rec + i);
            const float di = pi.d;
            const int kn = a.kvois[i];
            const int *__restrict__ nb = a.indi + i;
            const unsigned *__restrict__ pk = a.pk + i;
            for (int w = 0; w < kn; w += UNR) {
                unsigned c[UNR];
                int j[UNR];
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    c[u] = (w + u < kn) ? __ldg(pk + (w + u) * ld) : kSkip;
                    j[u] = (w + u < kn) ? __ldg(nb + (w + u) * ld) : 0;
                }
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    if (c[u] == kSkip) continue;
                    const PosFF pj = ld_ff(a.rec + j[u]);
                    const float dj = pj.d;
                    const float sx = sep1(pi.hx, pi.lx, pj.hx, pj.lx, b.lh[0], b.ll[0], b.half[0], b.pd[0]);
                    const float sy = sep1(pi.hy, pi.ly, pj.hy, pj.ly, b.lh[1], b.ll[1], b.half[1], b.pd[1]);
                    const float sz = sep1(pi.hz, pi.lz, pj.hz, pj.lz, b.lh[2], b.ll[2], b.half[2], b.pd[2]);
                    const float y = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
                    const int kk = (int)(c[u] >> kDkBits);
                    const float dk = (float)(c[u] & ((1u << kDkBits) - 1)) * kDkInv;
                    const float4 e = kk >= kmin ? sforce[kk - kmin] : __ldg(t.force4 + kk);
                    const float P = fmaf(dk, e.y, e.x);
                    const float B = fmaf(dk, e.w, e.z);
                    const float ft = fmaf(P, y, B * (di + dj)) * y;
                    fx.fma_add(ft, sx);
                    fy.fma_add(ft, sy);
                    fz.fma_add(ft, sz);
                }
            }
        }
        a.fx[i] = fx.value64();
        a.fy[i] = fy.value64();
        a.fz[i] = fz.value64();
    }
}

// ---- fused force pass + integrator (mixed step) ---------------------------------------
// The force pass of step n followed, per atom, by the corrector of step n and the predictor
// of step n+1 (vv_atom): positions are read from a.pos / a.posff (neighbours of step n) and
// written to a.pos_nxt / a.posff_nxt, so no thread overwrites a position another thread is
// still gathering.  The integrator's FP64 work then runs on the FP64 pipe while other warps
// of the same kernel keep the FP32 pipes busy, and one pass over x, v and F disappears.
// MULTI: several table kinds (FPOTB of KPAIR(i,j) and KPAIR(j,i)); PF 0 or 1 then.
template <int UNR, int MINB, int PF, bool MULTI = false>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_vv(DevAtoms a, DevTables t, double th)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    if (i < a.n) {
        const int stat = a.statu[i];
        KSum fx, fy, fz;
        const DevBox &bb = a.box[a.boxid[i]];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const BoxF b = load_boxf(bb);
            const PosFF pi = ld_ff(a.rec + i);
            const float di = pi.d;
            if (MULTI) {
                const int ti = a.ityp[i] - 1;
                walk_pairs<UNR, (PF != 0)>(a.indi + i, a.pk + i, (size_t)a.ld, a.kvois[i], [&](int j, unsigned c) {
                    const PosFF pj = ld_ff(a.rec + j);
                    force_pair<true>(pi, pj, c, di, pj.d, ti, a.ityp[j] - 1, b, t, fx, fy, fz);
                });
            } else if (PF == 2) {
                force_loop_batched<UNR>(a, t, i, pi, di, b, fx, fy, fz);
            } else {
                walk_pairs<UNR, (PF != 0)>(a.indi + i, a.pk + i, (size_t)a.ld, a.kvois[i], [&](int j, unsigned c) {
                    const PosFF pj = ld_ff(a.rec + j);
                    force_pair<false>(pi, pj, c, di, pj.d, 0, 0, b, t, fx, fy, fz);
                });
            }
        }
        const double Fx = fx.value64(), Fy = fy.value64(), Fz = fz.value64();
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            dmax = vv_atom<true>(a, i, stat, bb, th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

// One box: the fused step kernel with the box constants as kernel parameters (bfp for the pair
// loop, bp for the integrator) instead of per-thread registers loaded from the box array; the
// same arithmetic in the same order as k_force32_vv<UNR, MINB, 2>, so bitwise the same results.
template <int UNR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_vv_sb(DevAtoms a, DevTables t, double th, DevBox bp,
                                                                BoxF bfp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    if (i < a.n) {
        const int stat = a.statu[i];
        KSum fx, fy, fz;
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const PosFF pi = ld_ff(a.rec + i);
            force_loop_batched<UNR>(a, t, i, pi, pi.d, bfp, fx, fy, fz);
        }
        const double Fx = fx.value64(), Fy = fy.value64(), Fz = fz.value64();
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            dmax = vv_atom<true>(a, i, stat, bp, th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

// The fused step kernel (single kind) on the fixed-point records; SB: one box, its constants and
// units as kernel parameters.
template <int UNR, int MINB, bool SB>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_vv_fix(DevAtoms a, DevTables t, double th, DevBox bp,
                                                                 float3 fup)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    if (i < a.n) {
        const int stat = a.statu[i];
        const bool act = (stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE;
        const int bi = SB ? 0 : a.boxid[i];
        KSum fx, fy, fz;
        if (act) {
            float fu[3];
            if (SB) {
                fu[0] = fup.x;
                fu[1] = fup.y;
                fu[2] = fup.z;
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) fu[k] = a.box[bi].fixu[k];
            }
            force_loop_fix<UNR>(a, t, i, __ldg(a.rec16 + i), fu, fx, fy, fz);
        }
        // the compensated sums finished in FP32 (one rounding, ~6e-8 of the force) and widened
        // once: two FP64 instructions fewer per component in the FP64-heavy epilogue
        const double Fx = (double)fx.value(), Fy = (double)fy.value(), Fz = (double)fz.value();
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if (act) {
            if (SB) dmax = vv_atom<true>(a, i, stat, bp, th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
            else dmax = vv_atom<true>(a, i, stat, a.box[bi], th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

// ---- cell-tile variants (single kind) ----------------------------------------------------
// The block's halo (built by k_halo after each list build: the atoms of every cell in the
// 27-cell stencils of the block's cells, as runs of consecutive sorted atoms) is staged in
// shared memory, one warp per run with coalesced loads, as two float4 arrays holding the
// two halves of each 32 B record (consecutive records fall on consecutive 16 B bank
// groups).  Every neighbour is then read from shared memory through its 16-bit halo
// position instead of being gathered through L1 per lane.  A block without a tile, or whose
// halo exceeds the launch's capacity `cap`, gathers from global memory as the other
// variants do.  The arithmetic per pair and its order are those of the other variants, so
// the results are bitwise the same.
// 16 B global -> shared copy that completes asynchronously (cp.async, cached in L2 only)
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ bool stage_halo(const DevAtoms &a, const PosFF *src, float4 *s_hi, float4 *s_lo, int cap)
{
    const int2 m = a.hmeta[blockIdx.x];
    const bool tiled = m.x >= 0 && m.y <= cap;
    if (tiled) {
        // every copy of the block is in flight before any is waited for
        const int2 *runs = a.hruns + (size_t)blockIdx.x * (kHaloRuns + 1);
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int r = w; r < m.x; r += kBlock / 32) {
            const int2 q = runs[r];
            const int len = runs[r + 1].y - q.y;
            for (int k = lane; k < len; k += 32) {
                const float4 *p = reinterpret_cast<const float4 *>(src + q.x + k);
                cp_async16(s_hi + q.y + k, p);
                cp_async16(s_lo + q.y + k, p + 1);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    __syncthreads();
    return tiled;
}

__device__ __forceinline__ PosFF smem_ff(const float4 *s_hi, const float4 *s_lo, int l)
{
    const float4 h = s_hi[l], o = s_lo[l];
    PosFF p;
    p.hx = h.x; p.hy = h.y; p.hz = h.z; p.d = h.w;
    p.lx = o.x; p.ly = o.y; p.lz = o.z; p.lw = o.w;
    return p;
}

// F'(rho) from rho (FS: -1/2 rho^-1/2; EAM: DFEMBD interpolated), single kind
template <int POT>
__device__ __forceinline__ float embed_slope32(const DevAtoms &a, const DevTables &t, float rho)
{
    float d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0f) d = -0.5f * rsqrtf(rho);
    } else if (rho > 0.0f) {
        const float sk = rho / t.rhodf + 1.0f;
        int kk = (int)(sk + 0.000001f);
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
        }
        const float2 e = __ldg(t.embd2 + kk);
        d = fmaf(sk - (float)kk, e.y, e.x);
    }
    return d;
}

// density sum over the list of atom i; idx: list entries (global atom or halo position),
// load(v): the position record of entry v (v < 0: any valid record, not accumulated)
template <int UNR, class Idx, class Load>
__device__ __forceinline__ float density_loop(const DevTables &t, const Idx *__restrict__ nb, unsigned *__restrict__ pk,
                                              size_t ld, int kn, const PosFF &pi, const BoxF &b, float rej, Load load)
{
    KSum racc;
    int jn[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) jn[u] = u < kn ? (int)__ldg(nb + u * ld) : -1;
    for (int w = 0; w < kn; w += UNR) {
        int j[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) j[u] = jn[u];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int sl = w + UNR + u;
            jn[u] = sl < kn ? (int)__ldg(nb + sl * ld) : -1;
        }
        PosFF p[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) p[u] = load(j[u]);
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            float dk = 0.0f;
            int kk = 0;
            const unsigned c = pair_index(pi, p[u], b, t, rej, dk, kk);
            if (j[u] >= 0) pk[(w + u) * ld] = c;
            const bool ok = j[u] >= 0 && c != kSkip;
            const float2 e = __ldg(t.dens2 + (ok ? kk : 0));
            if (ok) racc.add(fmaf(dk, e.y, e.x));   // a skipped slot adds nothing (not even 0)
        }
    }
    return racc.value();
}

template <int POT, int UNR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_density32t(DevAtoms a, DevTables t, int cap)
{
    extern __shared__ float4 s_halo[];
    float4 *s_hi = s_halo, *s_lo = s_halo + cap;
    const bool tiled = stage_halo(a, a.posff, s_hi, s_lo, cap);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int kn = a.kvois[i];
    unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {   // the force pass skips it
        a.den32[i] = 0.0f;
        store_rec(a, i, ld_ff(a.posff + i));          // d = 0
        return;
    }
    const BoxF b = load_boxf(a.box[a.boxid[i]]);
    const float rej = t.ru2h + 4.0f * sqrtf(t.ru2h) * b.dlmax + 1e-5f * t.ru2h;
    const PosFF pi = ld_ff(a.posff + i);
    float rho;
    if (tiled) {
        rho = density_loop<UNR>(t, a.lidx + i, pk, ld, kn, pi, b, rej,
                                [&](int v) { return smem_ff(s_hi, s_lo, v >= 0 ? v : 0); });
    } else {
        const PosFF *pf = a.posff;
        rho = density_loop<UNR>(t, a.indi + i, pk, ld, kn, pi, b, rej,
                                [&](int v) { return ld_ff(pf + (v >= 0 ? v : i)); });
    }
    const float d = embed_slope32<POT>(a, t, rho);
    a.den32[i] = d;
    PosFF r = pi;
    r.d = d;
    store_rec(a, i, r);
}

// force loop of the fused tile kernel: force_loop_batched with the neighbour records read
// from the staged halo
template <int UNR>
__device__ __forceinline__ void force_loop_tile(const DevAtoms &a, const DevTables &t, int i, const PosFF &pi,
                                                float di, const BoxF &b, const float4 *s_hi, const float4 *s_lo,
                                                KSum &fx, KSum &fy, KSum &fz)
{
    const unsigned short *__restrict__ nb = a.lidx + i;
    const unsigned *__restrict__ pk = a.pk + i;
    const size_t ld = (size_t)a.ld;
    const int kn = a.kvois[i];
    unsigned cn[UNR];
    int jn[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
        cn[u] = u < kn ? __ldg(pk + u * ld) : kSkip;
        jn[u] = u < kn ? (int)__ldg(nb + u * ld) : 0;
    }
    for (int w = 0; w < kn; w += UNR) {
        unsigned c[UNR];
        int j[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            c[u] = cn[u];
            j[u] = jn[u];
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int sl = w + UNR + u;
            cn[u] = sl < kn ? __ldg(pk + sl * ld) : kSkip;
            jn[u] = sl < kn ? (int)__ldg(nb + sl * ld) : 0;
        }
        PosFF pj[UNR];
        float4 e[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const unsigned row = c[u] == kSkip ? 0u : (c[u] >> kDkBits);
            pj[u] = smem_ff(s_hi, s_lo, j[u]);
            e[u] = __ldg(t.force4 + row);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (c[u] != kSkip) force_pair_e(pi, pj[u], c[u], di, pj[u].d, e[u], b, fx, fy, fz);
    }
}

// the fused step kernel (k_force32_vv, single kind) on cell tiles
template <int UNR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_force32_vv_t(DevAtoms a, DevTables t, double th, int cap)
{
    extern __shared__ float4 s_halo[];
    float4 *s_hi = s_halo, *s_lo = s_halo + cap;
    const bool tiled = stage_halo(a, a.rec, s_hi, s_lo, cap);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    if (i < a.n) {
        const int stat = a.statu[i];
        KSum fx, fy, fz;
        const DevBox &bb = a.box[a.boxid[i]];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const BoxF b = load_boxf(bb);
            const PosFF pi = ld_ff(a.rec + i);
            if (tiled) force_loop_tile<UNR>(a, t, i, pi, pi.d, b, s_hi, s_lo, fx, fy, fz);
            else force_loop_batched<UNR>(a, t, i, pi, pi.d, b, fx, fy, fz);
        }
        const double Fx = fx.value64(), Fy = fy.value64(), Fz = fz.value64();
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            dmax = vv_atom<true>(a, i, stat, bb, th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

// launch shape of the tile variants: halo capacity (atoms) and its shared memory
constexpr int kTileCapSmall = 2048;    // 64 KB: 3 blocks per SM
constexpr int kTileCapLarge = 2560;    // 80 KB: 2 blocks per SM

template <class K>
static int tile_smem(K kernel, int cap)
{
    const int bytes = cap * 2 * (int)sizeof(float4);
    cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return bytes;
}

// ---- TMA-streamed variant of the step kernel ----------------------------------------------
// The block's 256 atoms read their list slots from shared memory: one thread issues a 2D
// tensor copy (cp.async.bulk.tensor) of the (256 atoms x kTmaSlots slots) tile of INDI and of
// the packed indices per stage, double-buffered behind two mbarriers, so the coalesced list
// stream leaves the load/store path of the SM that the neighbour gathers keep busy.  Every
// wait is bounded: on expiry the block records kErrTimeout, waits (bounded again) for the
// copies it issued and skips its atoms' work.
constexpr int kTmaSlots = 8;
constexpr unsigned long long kWaitNs = 500000000ull;   // 0.5 s per wait
constexpr long kWaitSpinCap = 1L << 26;                // fallback bound on the polls

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// waits for the phase of `parity` to complete, for at most kWaitNs of wall time
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity)
{
    const unsigned long long t0 = global_ns();
    for (long it = 0; it < kWaitSpinCap; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

// Self-test of the bounded wait: one block waits on a barrier whose phase nothing completes;
// the wait runs out, the kernel records kErrTimeout and returns.
__global__ void k_wait_selftest(int *flags)
{
    __shared__ alignas(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&flags[kFlagErr], kErrTimeout);
}

int launch_wait_selftest(msmgb_ctx *c)
{
    k_wait_selftest<<<1, 32, 0, c->stream>>>(c->a.flags);
    c->launches += 1;
    return check_launch(c, "wait self-test");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y, unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

template <int UNR>
__global__ void __launch_bounds__(kBlock, 4)
    k_force32_vv_tma(DevAtoms a, DevTables t, double th, const __grid_constant__ CUtensorMap tm_indi,
                     const __grid_constant__ CUtensorMap tm_pk)
{
    __shared__ alignas(128) int s_indi[2][kTmaSlots][kBlock];
    __shared__ alignas(128) unsigned s_pk[2][kTmaSlots][kBlock];
    __shared__ alignas(8) unsigned long long bar[2];
    __shared__ int s_maxkn;
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * kBlock, i = i0 + tid;
    const bool in = i < a.n;
    const int stat = in ? a.statu[i] : 0;
    const bool act = in && (stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE;
    const int kn = act ? a.kvois[i] : 0;
    if (tid == 0) {
        s_maxkn = 0;
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    atomicMax(&s_maxkn, kn);
    __syncthreads();
    const int nstage = (s_maxkn + kTmaSlots - 1) / kTmaSlots;
    constexpr unsigned kStageBytes = 2u * kTmaSlots * kBlock * sizeof(int);
    if (tid == 0)
        for (int st = 0; st < 2 && st < nstage; ++st) {
            mbar_expect_tx(&bar[st], kStageBytes);
            tma_load_2d(&s_indi[st][0][0], &tm_indi, i0, st * kTmaSlots, &bar[st]);
            tma_load_2d(&s_pk[st][0][0], &tm_pk, i0, st * kTmaSlots, &bar[st]);
        }
    KSum fx, fy, fz;
    PosFF pi;
    BoxF b;
    if (act) {
        pi = ld_ff(a.rec + i);
        b = load_boxf(a.box[a.boxid[i]]);
    }
    bool bail = false;
    int st = 0;
    for (; st < nstage; ++st) {
        const int buf = st & 1;
        const bool ok = mbar_wait_bounded(&bar[buf], (unsigned)((st >> 1) & 1));
        bail = __syncthreads_or(!ok) != 0;
        if (bail) break;
#pragma unroll
        for (int u0 = 0; u0 < kTmaSlots; u0 += UNR) {
            unsigned c[UNR];
            int j[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int w = st * kTmaSlots + u0 + u;
                c[u] = w < kn ? s_pk[buf][u0 + u][tid] : kSkip;
                j[u] = c[u] != kSkip ? s_indi[buf][u0 + u][tid] : i;
            }
            PosFF pj[UNR];
            float4 e[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                pj[u] = ld_ff(a.rec + (c[u] != kSkip ? j[u] : (act ? i : 0)));
                e[u] = __ldg(t.force4 + (c[u] != kSkip ? (c[u] >> kDkBits) : 0u));
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (c[u] != kSkip) force_pair_e(pi, pj[u], c[u], pi.d, pj[u].d, e[u], b, fx, fy, fz);
        }
        __syncthreads();                              // every thread is done with this buffer
        if (tid == 0 && st + 2 < nstage) {
            mbar_expect_tx(&bar[buf], kStageBytes);
            tma_load_2d(&s_indi[buf][0][0], &tm_indi, i0, (st + 2) * kTmaSlots, &bar[buf]);
            tma_load_2d(&s_pk[buf][0][0], &tm_pk, i0, (st + 2) * kTmaSlots, &bar[buf]);
        }
    }
    if (bail) {
        // copies issued for stages st and st + 1 may still be in flight: wait for them
        // (bounded) before the block's shared memory goes away, record the timeout, skip the work
        for (int s2 = st; s2 < st + 2 && s2 < nstage; ++s2) mbar_wait_bounded(&bar[s2 & 1], (unsigned)((s2 >> 1) & 1));
        if (tid == 0) atomicOr(&a.flags[kFlagErr], kErrTimeout);
        return;
    }
    float dmax = 0.0f;
    if (in) {
        const double Fx = fx.value64(), Fy = fy.value64(), Fz = fz.value64();
        a.fx[i] = Fx;
        a.fy[i] = Fy;
        a.fz[i] = Fz;
        const double4_32a p = a.pos[i];
        if (act) {
            dmax = vv_atom<true>(a, i, stat, a.box[a.boxid[i]], th, true, Fx, Fy, Fz, p, a.pos_nxt, a.posff_nxt);
        } else {
            a.pos_nxt[i] = p;
            a.posff_nxt[i] = a.posff[i];
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

// Builds the two TMA descriptors once per context (driver entry point fetched at run time,
// no link-time dependency on the driver library).  Unavailable -> the variants are skipped.
int ensure_list_maps(msmgb_ctx *c)
{
    if (c->tm_state) return c->tm_state;
    c->tm_state = -1;
    if (!c->a.pk || (c->a.ld % 256) != 0) return -1;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return -1;
    }
    typedef CUresult (*Encode)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                               const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    Encode enc = (Encode)fn;
    const cuuint64_t dims[2] = {(cuuint64_t)c->a.ld, (cuuint64_t)c->p.mxkvois};
    const cuuint64_t strides[1] = {(cuuint64_t)c->a.ld * sizeof(int)};
    const cuuint32_t box[2] = {(cuuint32_t)kBlock, (cuuint32_t)kTmaSlots};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r1 = enc(&c->tm_indi, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, (void *)c->a.indi, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    CUresult r2 = enc(&c->tm_pk, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, (void *)c->a.pk, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    c->tm_state = (r1 == CUDA_SUCCESS && r2 == CUDA_SUCCESS) ? 1 : -1;
    return c->tm_state;
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

bool uses_tiles(const msmgb_ctx *c)
{
    return c->tab.ngroup == 1 && c->p.precision == MSMGB_PREC_MIXED &&
           ((c->tune_dens_unroll & 64) != 0 || (c->tune_fused >= 20 && c->tune_fused < 24));
}

// variant codes of the fused kernel: (neighbours in flight, minimum resident blocks), codes
// 6-11 the same six with the next slots of the list loaded one iteration ahead, 12-17 with
// in addition every gather of a batch issued before its arithmetic (force_loop_batched),
// 18-19 the TMA-streamed list (2 and 4 neighbours per batch; skipped without descriptors),
// 20-23 cell tiles (2/4 neighbours per batch x halo capacity 2048 / 2560 atoms);
// with several table kinds codes 0-3: 2/4 in flight x {plain, list prefetch}.  Codes + 32:
// codes 0-17 (several kinds: 0-3) in 128-thread blocks.
constexpr int kFusedVariants = 24;

template <int UNR, int MINB>
static void fused_tile(msmgb_ctx *c, double h, int cap)
{
    const int smem = tile_smem(k_force32_vv_t<UNR, MINB>, cap);
    k_force32_vv_t<UNR, MINB><<<nblk(c->n, kBlock), kBlock, smem, c->stream>>>(c->a, c->tab, h, cap);
}

constexpr int kFusedVariantsMulti = 4;

static void fused_variant(msmgb_ctx *c, int code, double h)
{
    // +32: the global-gather variants in 128-thread blocks (a finer last wave)
    const int bs = (code & 32) ? 128 : kBlock;
    code &= ~32;
    const int g = nblk(c->n, bs);
    const int g256 = nblk(c->n, kBlock);
    // variants tuned for one box or for the fixed-point records fall back to the same loop on
    // the box array / the 32 B records when the state no longer allows them
    if ((code & 64) && c->nbox != 1) code &= ~64;
    if ((code & 128) && !(c->a.fix_on && c->tab.ngroup == 1)) code &= ~128;
    if (code & 128) {      // fixed-point records: 128 + 12..17 (+64 one box)
        const bool sb = (code & 64) != 0;
        const DevBox &b0 = c->hbox[0];
        const float3 fu = make_float3(b0.fixu[0], b0.fixu[1], b0.fixu[2]);
#define MSMGB_FX(U, M)                                                                                         \
    do {                                                                                                       \
        if (sb) k_force32_vv_fix<U, M, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, b0, fu);                \
        else k_force32_vv_fix<U, M, false><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, b0, fu);                 \
    } while (0)
        switch (code & 63) {
        case 13: MSMGB_FX(4, 1); break;
        case 14: MSMGB_FX(2, 4); break;
        case 15: MSMGB_FX(4, 4); break;
        case 16: MSMGB_FX(2, 5); break;
        case 17: MSMGB_FX(4, 5); break;
        default: MSMGB_FX(2, 1); break;
        }
#undef MSMGB_FX
        return;
    }
    if (c->tab.ngroup > 1) {      // several table kinds: codes 0-3
        switch (code) {
        case 1: k_force32_vv<4, 1, 0, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
        case 2: k_force32_vv<2, 1, 1, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
        case 3: k_force32_vv<4, 1, 1, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
        default: k_force32_vv<2, 1, 0, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
        }
        return;
    }
    switch (code) {
    case 1: k_force32_vv<4, 1, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 2: k_force32_vv<2, 4, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 3: k_force32_vv<4, 4, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 4: k_force32_vv<2, 5, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 5: k_force32_vv<4, 5, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 6: k_force32_vv<2, 1, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 7: k_force32_vv<4, 1, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 8: k_force32_vv<2, 4, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 9: k_force32_vv<4, 4, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 10: k_force32_vv<2, 5, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 11: k_force32_vv<4, 5, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 12: k_force32_vv<2, 1, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 13: k_force32_vv<4, 1, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 14: k_force32_vv<2, 4, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 15: k_force32_vv<4, 4, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 16: k_force32_vv<2, 5, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 17: k_force32_vv<4, 5, 2><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
    case 18: k_force32_vv_tma<2><<<g256, kBlock, 0, c->stream>>>(c->a, c->tab, h, c->tm_indi, c->tm_pk); break;
    case 19: k_force32_vv_tma<4><<<g256, kBlock, 0, c->stream>>>(c->a, c->tab, h, c->tm_indi, c->tm_pk); break;
    case 20: fused_tile<2, 3>(c, h, kTileCapSmall); break;
    case 21: fused_tile<4, 3>(c, h, kTileCapSmall); break;
    case 22: fused_tile<2, 2>(c, h, kTileCapLarge); break;
    case 23: fused_tile<4, 2>(c, h, kTileCapLarge); break;
    // +64 (one box): 12-17 with the box constants as kernel parameters
    case 64 + 12: k_force32_vv_sb<2, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    case 64 + 13: k_force32_vv_sb<4, 1><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    case 64 + 14: k_force32_vv_sb<2, 4><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    case 64 + 15: k_force32_vv_sb<4, 4><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    case 64 + 16: k_force32_vv_sb<2, 5><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    case 64 + 17: k_force32_vv_sb<4, 5><<<g, bs, 0, c->stream>>>(c->a, c->tab, h, c->hbox[0], load_boxf(c->hbox[0])); break;
    default: k_force32_vv<2, 1, 0><<<g, bs, 0, c->stream>>>(c->a, c->tab, h); break;
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
    const bool multi = c->tab.ngroup > 1;
    const bool tma = !multi && ensure_list_maps(c) == 1;
    const bool tiles = !multi && enable_halo(c) == MSMGB_OK;
    std::vector<int> codes;
    for (int code = 0; code < (multi ? kFusedVariantsMulti : kFusedVariants); ++code) codes.push_back(code);
    for (int code = multi ? 0 : 6; code < (multi ? kFusedVariantsMulti : 18); ++code) codes.push_back(32 + code);
    if (!multi && c->nbox == 1)
        for (int code = 12; code < 18; ++code) {
            codes.push_back(64 + code);
            codes.push_back(64 + 32 + code);
        }
    if (!multi && c->a.fix_on)      // +128: the fixed-point records (+64 one box)
        for (int code = 12; code < 18; ++code) {
            codes.push_back(128 + code);
            codes.push_back(128 + 32 + code);
            if (c->nbox == 1) {
                codes.push_back(128 + 64 + code);
                codes.push_back(128 + 64 + 32 + code);
            }
        }
    for (int code : codes) {
        if ((code == 18 || code == 19) && !tma) continue;
        if (code >= 20 && code < 24 && !tiles) continue;
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            fused_variant(c, code, 0.0);
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (tune_log()) fprintf(stderr, "msmgb tune: n=%d fused variant %d: %.4f ms\n", c->n, code, ms / 3.0f);
        if (ms < best) { best = ms; bestc = code; }
    }
    c->tune_fused = bestc;
    c->tune_ms_fused = best / 3.0f;
    c->tuned_fused_n = c->n;
    c->halo_on = uses_tiles(c);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemsetAsync(c->a.maxdisp, 0, sizeof(unsigned long long), c->stream);
    return check_launch(c, "autotune fused");
}



// shared-memory table window of the persistent variants (rows [kmin, ntp))
static void smem_window(const msmgb_ctx *c, int bytes_per_row, int *kmin, int *cnt)
{
    const int budget = 48 * 1024 / bytes_per_row;
    *cnt = std::min(budget, c->tab.ntp);
    *kmin = c->tab.ntp - *cnt;
}

static int persistent_grid(const void *kernel, int smem)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, smem);
    return std::max(1, per) * std::max(1, sms);
}

template <int POT, int UNR, int MINB>
static void dens_tile(msmgb_ctx *c, int cap)
{
    const int smem = tile_smem(k_density32t<POT, UNR, MINB>, cap);
    k_density32t<POT, UNR, MINB><<<nblk(c->n, kBlock), kBlock, smem, c->stream>>>(c->a, c->tab, cap);
}

template <int POT, bool MULTI>
static void dens_variant(msmgb_ctx *c, int unr)
{
    // +128: the one-thread-per-atom variants in 128-thread blocks (a finer last wave)
    const int bs = (unr & 128) ? 128 : kBlock;
    unr &= ~128;
    const int g = nblk(c->n, bs);
    if (!MULTI && (unr & 256)) {      // table-assisted index (+16: list slots one batch ahead)
        float qm, rejs;
        if (!density_q_params(c, &qm, &rejs)) {   // RU too long for the positions' quantum
            dens_variant<POT, MULTI>(c, 2);
            return;
        }
        const bool pf = (unr & 16) != 0;
        // +512: one box, its constants as a kernel parameter
        const bool sb = (unr & 512) != 0 && c->nbox == 1;
        const QBox qb = qbox_of(c->hbox[0], qm);
        // the prefetch variants also exist for states whose boxes are all periodic in x, y, z
        bool per = true;
        for (const DevBox &bx : c->hbox) per = per && bx.ifpd[0] && bx.ifpd[1] && bx.ifpd[2];
#define MSMGB_DQ(U, M)                                                                                        \
    do {                                                                                                      \
        if (sb) {                                                                                             \
            if (pf && per)                                                                                    \
                k_density32q<POT, U, M, true, true, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb); \
            else if (pf)                                                                                      \
                k_density32q<POT, U, M, true, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb);     \
            else k_density32q<POT, U, M, false, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb);  \
        } else {                                                                                              \
            if (pf && per)                                                                                    \
                k_density32q<POT, U, M, true, false, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb); \
            else if (pf) k_density32q<POT, U, M, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb);  \
            else k_density32q<POT, U, M, false><<<g, bs, 0, c->stream>>>(c->a, c->tab, qm, rejs, qb);         \
        }                                                                                                     \
    } while (0)
        switch (unr & 7) {
        case 3: MSMGB_DQ(2, 5); break;
        case 4: MSMGB_DQ(4, 1); break;
        case 5: MSMGB_DQ(4, 4); break;
        default: MSMGB_DQ(2, 1); break;
        }
#undef MSMGB_DQ
        return;
    }
    if (!MULTI && (unr & 64)) {   // cell tiles: +16 the larger halo capacity
        const bool large = (unr & 16) != 0;
        if ((unr & 7) == 4) {
            if (large) dens_tile<POT, 4, 2>(c, kTileCapLarge);
            else dens_tile<POT, 4, 3>(c, kTileCapSmall);
        } else {
            if (large) dens_tile<POT, 2, 2>(c, kTileCapLarge);
            else dens_tile<POT, 2, 3>(c, kTileCapSmall);
        }
        return;
    }
    if (!MULTI && (unr & 8)) {
        int kmin, cnt;
        smem_window(c, (int)sizeof(float2), &kmin, &cnt);
        const int smem = cnt * (int)sizeof(float2);
        if ((unr & 7) == 1) {
            k_density32s<POT, 1><<<persistent_grid((const void *)k_density32s<POT, 1>, smem), kBlock, smem, c->stream>>>(c->a, c->tab, kmin, cnt);
        } else {
            k_density32s<POT, 2><<<persistent_grid((const void *)k_density32s<POT, 2>, smem), kBlock, smem, c->stream>>>(c->a, c->tab, kmin, cnt);
        }
        return;
    }
    if (unr & 16) {
        switch (unr & 7) {
        case 4: k_density32<POT, MULTI, 4, 1, true><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
        case 5: k_density32<POT, MULTI, 4, 6, true><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
        case 3: k_density32<POT, MULTI, 2, 6, true><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
        default: k_density32<POT, MULTI, 2, 1, true><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
        }
        return;
    }
    switch (unr & 7) {
    case 1: k_density32<POT, MULTI, 1, 1, false><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
    case 4: k_density32<POT, MULTI, 4, 1, false><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
    case 5: k_density32<POT, MULTI, 4, 6, false><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
    case 3: k_density32<POT, MULTI, 2, 6, false><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
    default: k_density32<POT, MULTI, 2, 1, false><<<g, bs, 0, c->stream>>>(c->a, c->tab); break;
    }
}

template <bool MULTI>
static void force_variant(msmgb_ctx *c, int unr)
{
    const int g = nblk(c->n, kBlock);
    if (!MULTI && (unr & 8)) {
        int kmin, cnt;
        smem_window(c, (int)sizeof(float4), &kmin, &cnt);
        const int smem = cnt * (int)sizeof(float4);
        if ((unr & 7) == 1) {
            k_force32s<1><<<persistent_grid((const void *)k_force32s<1>, smem), kBlock, smem, c->stream>>>(c->a, c->tab, kmin, cnt);
        } else {
            k_force32s<2><<<persistent_grid((const void *)k_force32s<2>, smem), kBlock, smem, c->stream>>>(c->a, c->tab, kmin, cnt);
        }
        return;
    }
    if (!MULTI && (unr & 128) && c->a.fix_on) {     // +128: the batched loop on the fixed-point records
        switch (unr & 7) {
        case 4: k_force32_fix<4, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 5: k_force32_fix<4, 6><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        case 3: k_force32_fix<2, 6><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        default: k_force32_fix<2, 1><<<g, kBlock, 0, c->stream>>>(c->a, c->tab); break;
        }
        return;
    }
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
    if (!c->a.pk) return set_err(c, MSMGB_ERR_ARG, "mixed passes need the pair-index buffer (set MIXED precision)");
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
    // +32 (force, single kind): and all gathers of a batch before its arithmetic;
    // +8: persistent grid with the table in shared memory (single kind only)
    const bool single = c->tab.ngroup == 1;
    // +64 (density, single kind): cell tiles (+16: larger halo capacity)
    // +128: 128-thread blocks
    // +256 (single kind): table-assisted index (k_density32q), 2/4 in flight, registers capped
    // for 5 (2 in flight) or 4 (4 in flight) blocks of 256 threads, prefetch, 128-thread blocks
    std::vector<int> dc = {1, 2, 4, 3, 5, 18, 20, 19, 21, 131, 133, 147, 149};
    if (single) {
        dc.push_back(9);
        dc.push_back(10);
        if (enable_halo(c) == MSMGB_OK)
            for (int v : {66, 68, 82, 84}) dc.push_back(v);
        float qm, rejs;
        const bool q_ok = density_q_params(c, &qm, &rejs);
        for (int v : {258, 259, 260, 261, 274, 275, 276, 277, 386, 387, 388, 389, 402, 403, 404, 405}) {
            if (!q_ok) break;
            dc.push_back(v);
            if (c->nbox == 1) dc.push_back(512 + v);      // box constants as a kernel parameter
        }
    }
    // +128 (single kind): the batched loop on the fixed-point records
    std::vector<int> fcands = {1, 2, 4, 3, 5, 18, 20, 19, 21};
    if (single) {
        for (int v : {50, 52, 51, 53, 9, 10}) fcands.push_back(v);
        if (c->a.fix_on)
            for (int v : {50, 52, 51, 53}) fcands.push_back(128 + v);
    }
    const bool log = tune_log();
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err != cudaSuccess) return cuda_err(c, err, "autotune events");
    float best_d = 1e30f, best_f = 1e30f;
    int bd = 2, bf = 2;
    for (int code : dc) {
        c->tune_dens_unroll = code;
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            int rc = launch_density32(c);
            if (rc) return rc;
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (log) fprintf(stderr, "msmgb tune: n=%d density variant %d: %.4f ms\n", c->n, code, ms / 3.0f);
        if (ms < best_d) { best_d = ms; bd = code; }
    }
    c->tune_dens_unroll = bd;
    int rc = launch_density32(c);
    if (rc) return rc;
    for (size_t k = 0; k < fcands.size(); ++k) {
        c->tune_force_unroll = fcands[k];
        for (int r = 0; r < 4; ++r) {
            if (r == 1) cudaEventRecord(e0, c->stream);
            rc = launch_force32(c);
            if (rc) return rc;
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (log) fprintf(stderr, "msmgb tune: n=%d force variant %d: %.4f ms\n", c->n, fcands[k], ms / 3.0f);
        if (ms < best_f) { best_f = ms; bf = fcands[k]; }
    }
    c->tune_force_unroll = bf;
    c->tune_ms[0] = best_d / 3.0f;
    c->tune_ms[1] = best_f / 3.0f;
    c->tuned_n = c->n;
    c->halo_on = uses_tiles(c);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return check_launch(c, "autotune");
}

}  // namespace msmgb
