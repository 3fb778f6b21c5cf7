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
// The density pass is recomputed (nothing is kept from an earlier force call); its pair
// geometry (separation, 1/R, SK) is handed to the second pass through per-pair buffers in
// the list's ELL layout, so the second pass reads no positions and evaluates no square
// roots or image shifts.
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

template <int POT, bool MULTI>
__global__ void __launch_bounds__(kBlock) k_hvp_density(DevAtoms a, DevTables t, const double4_32a *v,
                                                        double2 *dd, double4_32a *pg, double *psk)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) {
        dd[i] = make_double2(0.0, 0.0);
        return;
    }
    // box parameters in registers: the per-pair stores below could alias the box array
    const DevBox &b = a.box[a.boxid[i]];
    const double lx = b.len[0], ly = b.len[1], lz = b.len[2];
    const double hx = b.half[0], hy = b.half[1], hz = b.half[2];
    const int px = b.ifpd[0], py = b.ifpd[1], pz = b.ifpd[2];
    const double4_32a p = a.pos[i];
    const double4_32a vi = v[i];
    const int ti = a.ityp[i] - 1;
    const int kn = a.kvois[i];
    const size_t ld = (size_t)a.ld;
    double rho = 0.0, rhod = 0.0;
    for (int w = 0; w < kn; ++w) {
        int j = __ldg(a.indi + i + w * ld);
        double4_32a q = a.pos[j];
        double sx = mi(p.x - q.x, lx, hx, px);
        double sy = mi(p.y - q.y, ly, hy, py);
        double sz = mi(p.z - q.z, lz, hz, pz);
        double r2 = sx * sx + sy * sy + sz * sz;
        if (r2 > t.ru2) {
            pg[w * ld + i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);   // beyond RU: skipped later
            continue;
        }
        const int k = MULTI ? t.kpair[(a.ityp[j] - 1) * t.ngroup + ti] : 0;
        double y = rsqrt(r2);
        double sr = rsqrt(y);
        double sk = sr * t.csi;
        pg[w * ld + i] = make_double4_32a(sx, sy, sz, y);
        psk[w * ld + i] = sk;
        int kk = min((int)sk, t.ntab);
        double dk = sk - kk;
        double4_32a vj = v[j];
        const double sw = sx * (vi.x - vj.x) + sy * (vi.y - vj.y) + sz * (vi.z - vj.z);
        double val, sl;
        lerp2(t.potb + (size_t)k * t.ntp, kk, dk, &val, &sl);
        rho += val;
        // dSK/dR * Rdot = (CSI/2) sqrt(R) / R^2 * (s.w); CSI/2 is applied once below
        rhod += sl * (sr * (y * y)) * sw;
    }
    rhod *= 0.5 * t.csi;
    double d = 0.0, ddot = 0.0;
    if (POT == MSMGB_FS_TYPE) {
        if (rho > 0.0) {
            double s = sqrt(rho);
            d = -0.5 / s;
            ddot = 0.25 * rhod / (rho * s);
        }
    } else if (rho > 0.0) {
        const double *T = t.dfembd + (size_t)(MULTI ? t.kembd[ti] : 0) * t.nep;
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
    dd[i] = make_double2(d, ddot);
}

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_hvp_force(DevAtoms a, DevTables t, const double4_32a *v,
                                                      const double2 *dd, const double4_32a *pg,
                                                      const double *psk, double *hx, double *hy, double *hz)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double gx = 0.0, gy = 0.0, gz = 0.0;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const double4_32a vi = v[i];
        const int ti = MULTI ? a.ityp[i] - 1 : 0;
        const double2 e_i = dd[i];
        const double di = e_i.x, ddi = e_i.y;
        const int kn = a.kvois[i];
        const size_t ld = (size_t)a.ld;
        for (int w = 0; w < kn; ++w) {
            // separation, 1/R and SK of the first pass (1/R = 0 beyond RU): the second pass
            // needs neither the positions nor square roots
            const double4_32a g = pg[w * ld + i];
            if (g.w == 0.0) continue;
            const int j = __ldg(a.indi + i + w * ld);
            const double sx = g.x, sy = g.y, sz = g.z, y = g.w;
            const double sk = psk[w * ld + i];
            int kk = min((int)sk, t.ntab);
            double dk = sk - kk;
            double skr = 0.5 * sk * y;      // dSK/dR = CSI / (2 sqrt(R)) = SK / (2 R)
            double4_32a vj = v[j];
            double wx = vi.x - vj.x, wy = vi.y - vj.y, wz = vi.z - vj.z;
            double rdot = (sx * wx + sy * wy + sz * wz) * y;
            const double2 e_j = dd[j];
            const double dj = e_j.x, ddj = e_j.y;
            double ft, ftd;
            if (!MULTI) {
                double P, Ps, B, Bs;
                const int k = 0;
                lerp2(t.fpotr + (size_t)k * t.ntp, kk, dk, &P, &Ps);
                lerp2(t.fpotb + (size_t)k * t.ntp, kk, dk, &B, &Bs);
                const double dsum = di + dj;
                const double emb = B * dsum;
                const double py_ = P * y;
                ft = (py_ + emb) * y;
                // dFT/dR = y (skr (Ps y + Bs dsum) - y (2 P y + emb))
                const double dft = y * (skr * (Ps * y + Bs * dsum) - y * (2.0 * py_ + emb));
                ftd = dft * rdot + B * (ddi + ddj) * y;
            } else {
                int tj = a.ityp[j] - 1;
                int k = t.kpair[tj * t.ngroup + ti];
                int k1 = t.kpair[ti * t.ngroup + tj];
                double P, Ps, B, Bs, B1, B1s;
                lerp2(t.fpotr + (size_t)k * t.ntp, kk, dk, &P, &Ps);
                lerp2(t.fpotb + (size_t)k * t.ntp, kk, dk, &B, &Bs);
                lerp2(t.fpotb + (size_t)k1 * t.ntp, kk, dk, &B1, &B1s);
                double y2 = y * y;
                double emb = B * di + B1 * dj;
                ft = P * y2 + emb * y;
                double dft = (Ps * skr) * y2 - 2.0 * P * y2 * y + (Bs * di + B1s * dj) * skr * y - emb * y2;
                ftd = dft * rdot + (B * ddi + B1 * ddj) * y;
            }
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
    if (!c->hvp_pair) return set_err(c, MSMGB_ERR_ARG, "HVP pair buffer not allocated");
    double4_32a *pg = (double4_32a *)c->hvp_pair;
    double *psk = (double *)(pg + (size_t)c->a.ld * (size_t)c->p.mxkvois);
    const int n = c->n;
    const int bs = block_for(n), g = nblk(n, bs);
    const bool multi = c->tab.ngroup > 1;
    double4_32a *v4 = (double4_32a *)v4buf;
    double2 *dd2 = (double2 *)ddbuf;
    k_gather_v<<<g, bs, 0, c->stream>>>(dv, c->a.gid, n, v4);
    if (c->tab.pottype == MSMGB_FS_TYPE) {
        if (multi) k_hvp_density<MSMGB_FS_TYPE, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk);
        else k_hvp_density<MSMGB_FS_TYPE, false><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk);
    } else {
        if (multi) k_hvp_density<MSMGB_EAM_TYPE, true><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk);
        else k_hvp_density<MSMGB_EAM_TYPE, false><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk);
    }
    if (multi) k_hvp_force<true><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk, dhv, dhv + n, dhv + 2 * (size_t)n);
    else k_hvp_force<false><<<g, bs, 0, c->stream>>>(c->a, c->tab, v4, dd2, pg, psk, dhv, dhv + n, dhv + 2 * (size_t)n);
    c->launches += 3;
    return check_launch(c, "hvp");
}

}  // namespace msmgb
