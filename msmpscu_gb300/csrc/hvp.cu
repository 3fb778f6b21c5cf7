// hvp.cu -- Hessian-vector product of the table-mode many-body force, FP64.
//
// No counterpart exists in the reference: its ART method pushes along the displacement
// and projects the force on the host (MD_Method_ART_GPU.F90:457-466, 570-576) and any
// curvature would need finite-difference force pairs.  This is the forward-over-reverse
// derivative of the force actually computed by the density and force passes (so it is
// exact for the piecewise-linear table interpolants):
//   pass 1 (k_hvp_density): rho_i, F'_i as in PRECALFOR_KERNEL and the directional
//     derivatives  rhodot_i = sum_j dPOTB(KK) dSK/dR Rdot_ij,  Rdot = s.(v_i - v_j)/R,
//     dSK/dR = CSI/(2 sqrt(R));  FS: F'dot = rho^(-3/2) rhodot / 4;
//     EAM: F'dot = dDFEMBD(KK) rhodot / RHOD.
//   pass 2 (k_hvp_force): Fdot_i = sum_j FTdot s + FT (v_i - v_j) with
//     FT = P/R^2 + (B F'_i + B1 F'_j)/R,
//     dFT/dR = P'/R^2 - 2P/R^3 + (B' F'_i + B1' F'_j)/R - (B F'_i + B1 F'_j)/R^2,
//     FTdot = dFT/dR Rdot + (B F'dot_i + B1 F'dot_j)/R;   hv = -Fdot.
// The density pass is recomputed (not stored), so the product costs two passes like a
// force call.
#include "msmgb_internal.cuh"

namespace msmgb {

__device__ __forceinline__ double mi(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

__device__ __forceinline__ void lerp2(const double *__restrict__ T, int kk, double dk, double *val,
                                      double *slope)
{
    double a = __ldg(T + kk), b = __ldg(T + kk + 1);
    *slope = b - a;
    *val = a + dk * (b - a);
}

template <int POT>
__global__ void __launch_bounds__(kBlock) k_hvp_density(DevAtoms a, DevTables t, const double4_32a *v,
                                                        double *dd)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        a.den[i] = 0.0;
        dd[i] = 0.0;
        return;
    }
    const DevBox &b = a.box[a.boxid[i]];
    const double4_32a p = a.pos[i];
    const double4_32a vi = v[i];
    const int ti = a.ityp[i] - 1;
    const int kn = a.kvois[i];
    const size_t ld = (size_t)a.ld;
    double rho = 0.0, rhod = 0.0;
    for (int w = 0; w < kn; ++w) {
        int j = __ldg(a.indi + i + w * ld);
        double4_32a q = a.pos[j];
        double sx = mi(p.x - q.x, b.len[0], b.half[0], b.ifpd[0]);
        double sy = mi(p.y - q.y, b.len[1], b.half[1], b.ifpd[1]);
        double sz = mi(p.z - q.z, b.len[2], b.half[2], b.ifpd[2]);
        double r2 = sx * sx + sy * sy + sz * sz;
        if (r2 > t.ru2) continue;
        int k = t.kpair[(a.ityp[j] - 1) * t.ngroup + ti];
        double y = rsqrt(r2);
        double sr = rsqrt(y);
        double sk = sr * t.csi;
        int kk = min((int)sk, t.ntab);
        double dk = sk - kk;
        double4_32a vj = v[j];
        double rdot = (sx * (vi.x - vj.x) + sy * (vi.y - vj.y) + sz * (vi.z - vj.z)) * y;
        double val, sl;
        lerp2(t.potb + (size_t)k * t.ntp, kk, dk, &val, &sl);
        rho += val;
        rhod += sl * (0.5 * t.csi * y * sr) * rdot;      // dSK/dR = CSI / (2 sqrt(R))
    }
    double d = 0.0, ddot = 0.0;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0) {
            double s = sqrt(rho);
            d = -0.5 / s;
            ddot = 0.25 * rhod / (rho * s);
        }
    } else if (rho > 0.0) {
        const double *T = t.dfembd + (size_t)t.kembd[ti] * t.nep;
        double sk = rho / t.rhod + 1.0;
        int kk = (int)(sk + 0.000001);
        if (kk + 1 > t.nembd) {
            atomicOr(&a.flags[kFlagErr], kErrRho);
            kk = t.nembd;
        }
        double e0 = __ldg(T + kk), e1 = __ldg(T + kk + 1);
        d = e0 + (sk - kk) * (e1 - e0);
        ddot = (e1 - e0) * rhod / t.rhod;
    } else {
        d = rho;
    }
    a.den[i] = d;
    dd[i] = ddot;
}

__global__ void __launch_bounds__(kBlock) k_hvp_force(DevAtoms a, DevTables t, const double4_32a *v,
                                                      const double *dd, double *hx, double *hy, double *hz)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double gx = 0.0, gy = 0.0, gz = 0.0;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &b = a.box[a.boxid[i]];
        const double4_32a p = a.pos[i];
        const double4_32a vi = v[i];
        const int ti = a.ityp[i] - 1;
        const double di = a.den[i], ddi = dd[i];
        const int kn = a.kvois[i];
        const size_t ld = (size_t)a.ld;
        for (int w = 0; w < kn; ++w) {
            int j = __ldg(a.indi + i + w * ld);
            double4_32a q = a.pos[j];
            double sx = mi(p.x - q.x, b.len[0], b.half[0], b.ifpd[0]);
            double sy = mi(p.y - q.y, b.len[1], b.half[1], b.ifpd[1]);
            double sz = mi(p.z - q.z, b.len[2], b.half[2], b.ifpd[2]);
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 > t.ru2) continue;
            int tj = a.ityp[j] - 1;
            int k = t.kpair[tj * t.ngroup + ti];
            int k1 = t.kpair[ti * t.ngroup + tj];
            double y = rsqrt(r2);           // 1/R
            double sr = rsqrt(y);           // sqrt(R)
            double sk = sr * t.csi;
            int kk = min((int)sk, t.ntab);
            double dk = sk - kk;
            double skr = 0.5 * t.csi * y * sr;
            double4_32a vj = v[j];
            double wx = vi.x - vj.x, wy = vi.y - vj.y, wz = vi.z - vj.z;
            double rdot = (sx * wx + sy * wy + sz * wz) * y;
            double dj = a.den[j], ddj = dd[j];
            double P, Ps, B, Bs, B1, B1s;
            lerp2(t.fpotr + (size_t)k * t.ntp, kk, dk, &P, &Ps);
            lerp2(t.fpotb + (size_t)k * t.ntp, kk, dk, &B, &Bs);
            if (k1 != k) lerp2(t.fpotb + (size_t)k1 * t.ntp, kk, dk, &B1, &B1s);
            else { B1 = B; B1s = Bs; }
            double y2 = y * y;
            double emb = B * di + B1 * dj;
            double ft = P * y2 + emb * y;
            double dft = (Ps * skr) * y2 - 2.0 * P * y2 * y + (Bs * di + B1s * dj) * skr * y - emb * y2;
            double ftd = dft * rdot + (B * ddi + B1 * ddj) * y;
            gx += ftd * sx + ft * wx;
            gy += ftd * sy + ft * wy;
            gz += ftd * sz + ft * wz;
        }
    }
    hx[i] = -gx;
    hy[i] = -gy;
    hz[i] = -gz;
}

// v (caller order, XP layout) -> sorted double4
__global__ void k_gather_v(const double *src, const int *gid, int n, double4_32a *dst)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int g = gid[s];
    dst[s] = make_double4_32a(src[g], src[n + g], src[2 * n + g], 0.0);
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

// dv: caller-order XP layout on the device; dhv: sorted SoA output (3 slabs of n)
int launch_hvp(msmgb_ctx *c, const double *dv, double *dhv, double *v4buf, double *ddbuf)
{
    const int n = c->n;
    double4_32a *v4 = (double4_32a *)v4buf;
    k_gather_v<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(dv, c->a.gid, n, v4);
    if (c->tab.pottype == MSMGB_FS_TYPE)
        k_hvp_density<MSMGB_FS_TYPE><<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a, c->tab, v4, ddbuf);
    else
        k_hvp_density<MSMGB_EAM_TYPE><<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a, c->tab, v4, ddbuf);
    k_hvp_force<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a, c->tab, v4, ddbuf, dhv, dhv + n,
                                                         dhv + 2 * (size_t)n);
    c->launches += 3;
    return check_launch(c, "hvp");
}

}  // namespace msmgb
