// force64.cu -- plain FP64 force passes (the reference's arithmetic).
//
//   k_density64  PRECALFOR_KERNEL  (FS: MD_FS_ForceTable_GPU.F90:341-516,
//                                   EAM: MD_EAM_ForceTable_GPU.F90:369-548)
//                rho_i = sum_j POTB(SK), SK = sqrt(R) CSI; FS: F'_i = -1/(2 sqrt(rho_i)),
//                EAM: F'_i = DFEMBD(rho_i / RHOD + 1); with EPOT also CALEPOT_KERNEL
//                (:1451-1609 / :1470-1636): E_i = sum_j POTR(SK)/R + F(rho_i).
//   k_force64    CALFORCE_KERNEL / CALPTENSOR_KERNEL (:623-806, :998-1272 and EAM twins)
//                FORTOT = FPOTR/R^2 + (FPOTB(k_ij) F'_i + FPOTB(k_ji) F'_j)/R,
//                F_i = sum_j FORTOT s_ij, virial P_ab += FORTOT/2 s_a s_b per box.
//   k_stress64   CAL_FS_AtomicStress_KERNEL / CAL_EAM_AtomicStress_KERNEL
//                (MD_FS_ForceTable_GPU.F90:1746-1965, MD_EAM_ForceTable_GPU.F90:1775-1994)
//                AP_i(a,b) = sum_j FORTOT s_a s_b, written straight into the caller's order.
//
// One thread per atom over the cell-sorted order, so the 32 atoms of a warp share most of
// their neighbours and the double4_32a position gathers hit L1/L2.  The two square roots and
// the two divisions of the reference per pair are replaced by two reciprocal square
// roots (1/R = rsqrt(R^2), sqrt(R) = rsqrt(1/R)); the results differ from the reference's
// expression by a few ulp.  These passes are bound by the FP64 pipe on GB300.
#include "msmgb_internal.cuh"

namespace msmgb {

__device__ __forceinline__ double mi(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

// T(KK) + DK (T(KK+1) - T(KK)) on a padded row (entries 0 .. ntab+1)
__device__ __forceinline__ double lerp_row(const double *__restrict__ T, int kk, double dk)
{
    double a = __ldg(T + kk), b = __ldg(T + kk + 1);
    return a + dk * (b - a);
}

template <bool MULTI>
__device__ __forceinline__ int pair_kind(const DevTables &t, int ti, int tj)
{
    return MULTI ? t.kpair[tj * t.ngroup + ti] : 0;
}

// EAM embedding lookup (MD_EAM_ForceTable_GPU.F90:535-541): SK = rho/RHOD + 1,
// KK = int(SK + 1e-6), 1-based; rows are padded so index nembd+1 is readable.
__device__ __forceinline__ double embed_lookup(const double *__restrict__ T, int nembd, double rho,
                                               double rhod, int *flags)
{
    double sk = rho / rhod + 1.0;
    int kk = (int)(sk + 0.000001);
    if (kk + 1 > nembd) {
        atomicOr(&flags[kFlagErr], kErrRho);
        kk = nembd;
    }
    if (kk < 0) kk = 0;
    double a = __ldg(T + kk), b = __ldg(T + kk + 1);
    return a + (sk - kk) * (b - a);
}

template <int POT, bool MULTI, bool EPOT, bool SHAPED = false>
__global__ void __launch_bounds__(kBlock) k_density64(DevAtoms a, DevTables t)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        a.den[i] = 0.0;
        if (EPOT) a.epot[i] = 0.0;
        return;
    }
    const DevBox &b = a.box[a.boxid[i]];
    const double lx = b.len[0], ly = b.len[1], lz = b.len[2];
    const double hx = b.half[0], hy = b.half[1], hz = b.half[2];
    const int px = b.ifpd[0], py = b.ifpd[1], pz = b.ifpd[2];
    const double4_32a p = a.pos[i];
    const int ti = MULTI ? a.ityp[i] - 1 : 0;
    const int kn = a.kvois[i];
    const int *__restrict__ nb = a.indi + i;
    const size_t ld = (size_t)a.ld;
    double rho = 0.0, er = 0.0;
    for (int w = 0; w < kn; ++w) {
        int j = __ldg(nb + w * ld);
        double4_32a q = a.pos[j];
        double sx = mi(p.x - q.x, lx, hx, px);
        double sy = mi(p.y - q.y, ly, hy, py);
        double sz = mi(p.z - q.z, lz, hz, pz);
        if (SHAPED) shape_sep(b, sx, sy, sz);   // a state with a non-cubic box
        double r2 = sx * sx + sy * sy + sz * sz;
        if (r2 <= t.ru2) {
            int k = pair_kind<MULTI>(t, ti, MULTI ? a.ityp[j] - 1 : 0);
            double y = rsqrt(r2);          // 1/R
            double sr = rsqrt(y);          // sqrt(R)
            double sk = sr * t.csi;
            int kk = min((int)sk, t.ntab);
            double dk = sk - kk;
            rho += lerp_row(t.potb + (size_t)k * t.ntp, kk, dk);
            if (EPOT) er += lerp_row(t.potr + (size_t)k * t.ntp, kk, dk) * y;
        }
    }
    double d = rho;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0) d = -0.5 / sqrt(rho);
        if (EPOT) a.epot[i] = er - sqrt(rho);
    } else {
        const int ke = MULTI ? t.kembd[ti] : 0;
        if (rho > 0.0) d = embed_lookup(t.dfembd + (size_t)ke * t.nep, t.nembd, rho, t.rhod, a.flags);
        if (EPOT) a.epot[i] = er + embed_lookup(t.fembd + (size_t)ke * t.nep, t.nembd, rho, t.rhod, a.flags);
    }
    a.den[i] = d;
}

// per-box virial accumulation: warp-uniform boxes reduce in registers, then one atomic
__device__ __forceinline__ void virial_flush(DevAtoms &a, int box, double v[6])
{
    const unsigned full = 0xffffffffu;
    int b0 = __shfl_sync(full, box, 0);
    bool uniform = __all_sync(full, box == b0 || box < 0);
    if (uniform) {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            double x = v[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(full, x, o);
            v[c] = x;
        }
        if ((threadIdx.x & 31) == 0 && b0 >= 0)
            for (int c = 0; c < 6; ++c) atomicAdd(&a.virial[b0 * 6 + c], v[c]);
    } else if (box >= 0) {
        for (int c = 0; c < 6; ++c) atomicAdd(&a.virial[box * 6 + c], v[c]);
    }
}

template <int POT, bool MULTI, bool VIRIAL, bool SHAPED = false>
__global__ void __launch_bounds__(kBlock) k_force64(DevAtoms a, DevTables t)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    double v[6] = {0, 0, 0, 0, 0, 0};
    int box = -1;
    if (i < a.n && (a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        box = a.boxid[i];
        const DevBox &b = a.box[box];
        const double lx = b.len[0], ly = b.len[1], lz = b.len[2];
        const double hx = b.half[0], hy = b.half[1], hz = b.half[2];
        const int px = b.ifpd[0], py = b.ifpd[1], pz = b.ifpd[2];
        const double4_32a p = a.pos[i];
        const int ti = MULTI ? a.ityp[i] - 1 : 0;
        const double di = a.den[i];
        const int kn = a.kvois[i];
        const int *__restrict__ nb = a.indi + i;
        const size_t ld = (size_t)a.ld;
        for (int w = 0; w < kn; ++w) {
            int j = __ldg(nb + w * ld);
            double4_32a q = a.pos[j];
            double sx = mi(p.x - q.x, lx, hx, px);
            double sy = mi(p.y - q.y, ly, hy, py);
            double sz = mi(p.z - q.z, lz, hz, pz);
            if (SHAPED) shape_sep(b, sx, sy, sz);   // a state with a non-cubic box
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 <= t.ru2) {
                int tj = MULTI ? a.ityp[j] - 1 : 0;
                int k = pair_kind<MULTI>(t, ti, tj);
                int k1 = pair_kind<MULTI>(t, tj, ti);
                double y = rsqrt(r2);
                double sr = rsqrt(y);
                double sk = sr * t.csi;
                int kk = min((int)sk, t.ntab);
                double dk = sk - kk;
                double dj = a.den[j];
                const double *rowb = t.fpotb + (size_t)k * t.ntp;
                double P = lerp_row(t.fpotr + (size_t)k * t.ntp, kk, dk);
                double B = lerp_row(rowb, kk, dk);
                double B1 = (MULTI && k1 != k) ? lerp_row(t.fpotb + (size_t)k1 * t.ntp, kk, dk) : B;
                double ft = P * (y * y) + (B * di + B1 * dj) * y;
                fx += ft * sx;
                fy += ft * sy;
                fz += ft * sz;
                if (VIRIAL) {
                    double hf = ft * 0.5;
                    v[0] += sx * sx * hf; v[1] += sx * sy * hf; v[2] += sx * sz * hf;
                    v[3] += sy * sy * hf; v[4] += sy * sz * hf; v[5] += sz * sz * hf;
                }
            }
        }
    }
    if (i < a.n) {
        a.fx[i] = fx;
        a.fy[i] = fy;
        a.fz[i] = fz;
    }
    if (VIRIAL) virial_flush(a, box, v);
}

// Per-atom virial tensor from the F'(rho) of the last FP64 density pass.  ap holds 9 slabs
// of n doubles (component 3a+b, the reference's AP(NAPDEV, 9)); atom i goes to row gid[i]
// (caller order) or i (sorted order).
template <bool MULTI, bool SHAPED = false>
__global__ void __launch_bounds__(kBlock) k_stress64(DevAtoms a, DevTables t, int sorted, double *ap)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double p[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &b = a.box[a.boxid[i]];
        const double4_32a pi = a.pos[i];
        const int ti = MULTI ? a.ityp[i] - 1 : 0;
        const double di = a.den[i];
        const int kn = a.kvois[i];
        const size_t ld = (size_t)a.ld;
        for (int w = 0; w < kn; ++w) {
            const int j = __ldg(a.indi + i + w * ld);
            const double4_32a q = a.pos[j];
            double s[3];
            s[0] = mi(pi.x - q.x, b.len[0], b.half[0], b.ifpd[0]);
            s[1] = mi(pi.y - q.y, b.len[1], b.half[1], b.ifpd[1]);
            s[2] = mi(pi.z - q.z, b.len[2], b.half[2], b.ifpd[2]);
            if (SHAPED) shape_sep(b, s[0], s[1], s[2]);
            const double r2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
            if (r2 > t.ru2) continue;
            const int tj = MULTI ? a.ityp[j] - 1 : 0;
            const int k = pair_kind<MULTI>(t, ti, tj);
            const int k1 = pair_kind<MULTI>(t, tj, ti);
            const double y = rsqrt(r2);
            const double sk = rsqrt(y) * t.csi;
            const int kk = min((int)sk, t.ntab);
            const double dk = sk - kk;
            const double P = lerp_row(t.fpotr + (size_t)k * t.ntp, kk, dk);
            const double B = lerp_row(t.fpotb + (size_t)k * t.ntp, kk, dk);
            const double B1 = (MULTI && k1 != k) ? lerp_row(t.fpotb + (size_t)k1 * t.ntp, kk, dk) : B;
            const double ft = P * (y * y) + (B * di + B1 * a.den[j]) * y;
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int v = 0; v < 3; ++v) p[3 * u + v] += s[u] * s[v] * ft;
        }
    }
    const size_t row = sorted ? (size_t)i : (size_t)a.gid[i];
#pragma unroll
    for (int m = 0; m < 9; ++m) ap[(size_t)m * a.n + row] = p[m];
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

template <int POT, bool MULTI>
static void dens_dispatch(msmgb_ctx *c, bool epot)
{
    const int bs = block_for(c->n), g = nblk(c->n, bs);
    if (c->any_shaped) {
        if (epot) k_density64<POT, MULTI, true, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_density64<POT, MULTI, false, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    } else {
        if (epot) k_density64<POT, MULTI, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_density64<POT, MULTI, false><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    }
}

template <int POT, bool MULTI>
static void force_dispatch(msmgb_ctx *c, bool vir)
{
    const int bs = block_for(c->n), g = nblk(c->n, bs);
    if (c->any_shaped) {
        if (vir) k_force64<POT, MULTI, true, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_force64<POT, MULTI, false, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    } else {
        if (vir) k_force64<POT, MULTI, true><<<g, bs, 0, c->stream>>>(c->a, c->tab);
        else k_force64<POT, MULTI, false><<<g, bs, 0, c->stream>>>(c->a, c->tab);
    }
}

int launch_density(msmgb_ctx *c, bool want_epot)
{
    bool multi = c->tab.ngroup > 1;
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) dens_dispatch<MSMGB_FS_TYPE, true>(c, want_epot);
        else dens_dispatch<MSMGB_FS_TYPE, false>(c, want_epot);
    } else {
        if (multi) dens_dispatch<MSMGB_EAM_TYPE, true>(c, want_epot);
        else dens_dispatch<MSMGB_EAM_TYPE, false>(c, want_epot);
    }
    c->launches += 1;
    c->den_is32 = false;
    return check_launch(c, "density pass");
}

int launch_stress(msmgb_ctx *c, int sorted, double *ap)
{
    const int bs = block_for(c->n), g = nblk(c->n, bs);
    if (c->any_shaped) {
        if (c->tab.ngroup > 1) k_stress64<true, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, sorted, ap);
        else k_stress64<false, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, sorted, ap);
    } else {
        if (c->tab.ngroup > 1) k_stress64<true><<<g, bs, 0, c->stream>>>(c->a, c->tab, sorted, ap);
        else k_stress64<false><<<g, bs, 0, c->stream>>>(c->a, c->tab, sorted, ap);
    }
    c->launches += 1;
    return check_launch(c, "atomic stress pass");
}

int launch_force(msmgb_ctx *c, bool want_virial)
{
    bool multi = c->tab.ngroup > 1;
    if (want_virial) {
        cudaError_t e = cudaMemsetAsync(c->a.virial, 0, sizeof(double) * 6 * (size_t)c->nbox, c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "virial clear");
    }
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) force_dispatch<MSMGB_FS_TYPE, true>(c, want_virial);
        else force_dispatch<MSMGB_FS_TYPE, false>(c, want_virial);
    } else {
        if (multi) force_dispatch<MSMGB_EAM_TYPE, true>(c, want_virial);
        else force_dispatch<MSMGB_EAM_TYPE, false>(c, want_virial);
    }
    c->launches += 1;
    return check_launch(c, "force pass");
}

}  // namespace msmgb
