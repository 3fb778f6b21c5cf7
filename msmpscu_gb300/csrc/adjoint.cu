// adjoint.cu -- gradient of a force-matching loss with respect to the potential parameters.
//
// No counterpart exists in the reference (it has no fitting code).  For the FS-type
// Cleri-Rosato tables and L = sum_i |F_i - Ft_i|^2, with w = F - Ft (zero on inactive
// atoms, whose force does not depend on the parameters) and, per pair,
// FT = P/R^2 + B (D_i + D_j)/R (P = FPOTR, B = FPOTB interpolated, D = -1/(2 sqrt(rho))):
//   dL/dtheta_m = 2 [ sum_i sum_j (w_i.s_ij) (dP_m/R^2 + dB_m (D_i + D_j)/R)
//                   + sum_i dD_i,m sum_j ((w_i - w_j).s_ij) B/R ]
//   dD_i,m = rho_i^(-3/2)/4 * sum_j dPOTB_m(r_ij)
// where dP_m, dB_m, dPOTB_m interpolate the parameter-derivative tables on the same grid
// (exact derivative of the table-mode force).  The second sum uses the symmetry of the full
// list (j in N(i) <=> i in N(j)).  Pass 1 recomputes rho (it is not stored from the force
// call), pass 2 accumulates the five components; both are FP64.
#include "msmgb_internal.cuh"

namespace msmgb {

struct AdjTables {
    const double *dfpotr[5];
    const double *dpotb[5];
    const double *dfpotb[5];
};

__device__ __forceinline__ double mi(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

__device__ __forceinline__ double lerp_row(const double *__restrict__ T, int kk, double dk)
{
    double a = __ldg(T + kk), b = __ldg(T + kk + 1);
    return a + dk * (b - a);
}

// block-wide sum of NV doubles, one atomicAdd per value and block
template <int NV>
__device__ __forceinline__ void block_sum_flush(double v[NV], double *dst)
{
    __shared__ double sm[NV][kBlock / 32];
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double x = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(full, x, o);
        if ((threadIdx.x & 31) == 0) sm[c][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm[threadIdx.x][w];
        atomicAdd(dst + threadIdx.x, s);
    }
}

__global__ void __launch_bounds__(kBlock) k_adj_residual(DevAtoms a, const double *ft, double4_32a *w,
                                                         double *acc)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    double l[1] = {0.0};
    if (s < a.n) {
        int g = a.gid[s], n = a.n;
        double rx = a.fx[s] - ft[g], ry = a.fy[s] - ft[n + g], rz = a.fz[s] - ft[2 * n + g];
        l[0] = rx * rx + ry * ry + rz * rz;
        bool act = (a.statu[s] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE;
        w[s] = act ? make_double4_32a(rx, ry, rz, 0.0) : make_double4_32a(0.0, 0.0, 0.0, 0.0);
    }
    block_sum_flush<1>(l, acc + 5);
}

__global__ void __launch_bounds__(kBlock) k_adj_density(DevAtoms a, DevTables t, AdjTables d, double *dd,
                                                        int cap)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double rho = 0.0, dr[5] = {0, 0, 0, 0, 0};
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &b = a.box[a.boxid[i]];
        const double4_32a p = a.pos[i];
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
            double y = rsqrt(r2);
            double sk = rsqrt(y) * t.csi;
            int kk = min((int)sk, t.ntab);
            double dk = sk - kk;
            rho += lerp_row(t.potb, kk, dk);
#pragma unroll
            for (int m = 0; m < 5; ++m) dr[m] += lerp_row(d.dpotb[m], kk, dk);
        }
    }
    double den = 0.0, c = 0.0;
    if (rho > 0.0) {
        double sr = sqrt(rho);
        den = -0.5 / sr;
        c = 0.25 / (rho * sr);
    }
    a.den[i] = den;
#pragma unroll
    for (int m = 0; m < 5; ++m) dd[(size_t)m * cap + i] = c * dr[m];
}

__global__ void __launch_bounds__(kBlock) k_adj_force(DevAtoms a, DevTables t, AdjTables d,
                                                      const double4_32a *w, const double *dd, int cap,
                                                      double *acc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double g[5] = {0, 0, 0, 0, 0};
    if (i < a.n && (a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const DevBox &b = a.box[a.boxid[i]];
        const double4_32a p = a.pos[i];
        const double4_32a wi = w[i];
        const double di = a.den[i];
        const int kn = a.kvois[i];
        const size_t ld = (size_t)a.ld;
        double cpl = 0.0;
        for (int ww = 0; ww < kn; ++ww) {
            int j = __ldg(a.indi + i + ww * ld);
            double4_32a q = a.pos[j];
            double sx = mi(p.x - q.x, b.len[0], b.half[0], b.ifpd[0]);
            double sy = mi(p.y - q.y, b.len[1], b.half[1], b.ifpd[1]);
            double sz = mi(p.z - q.z, b.len[2], b.half[2], b.ifpd[2]);
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 > t.ru2) continue;
            double y = rsqrt(r2);
            double sk = rsqrt(y) * t.csi;
            int kk = min((int)sk, t.ntab);
            double dk = sk - kk;
            double4_32a wj = w[j];
            double dj = a.den[j];
            double wis = wi.x * sx + wi.y * sy + wi.z * sz;
            double wd = (wi.x - wj.x) * sx + (wi.y - wj.y) * sy + (wi.z - wj.z) * sz;
            double B = lerp_row(t.fpotb, kk, dk);
            double dsum = (di + dj) * y;
            double y2 = y * y;
#pragma unroll
            for (int m = 0; m < 5; ++m)
                g[m] += wis * (lerp_row(d.dfpotr[m], kk, dk) * y2 + lerp_row(d.dfpotb[m], kk, dk) * dsum);
            cpl += wd * B * y;
        }
#pragma unroll
        for (int m = 0; m < 5; ++m) g[m] += dd[(size_t)m * cap + i] * cpl;
    }
    block_sum_flush<5>(g, acc);
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

// ft: caller-order target forces (XP layout) on the device; dtab: padded derivative rows
// [(m*3 + table)][ntp]; w4/dd: scratch; acc: 6 doubles (5 gradient sums + loss), zeroed here.
int launch_adjoint(msmgb_ctx *c, const double *ft, const double *dtab, double *w4buf, double *ddbuf,
                   double *acc)
{
    const int n = c->n;
    const size_t ntp = (size_t)c->tab.ntp;
    AdjTables d;
    for (int m = 0; m < 5; ++m) {
        d.dfpotr[m] = dtab + (size_t)(m * 3 + 0) * ntp;
        d.dpotb[m] = dtab + (size_t)(m * 3 + 1) * ntp;
        d.dfpotb[m] = dtab + (size_t)(m * 3 + 2) * ntp;
    }
    cudaError_t e = cudaMemsetAsync(acc, 0, 6 * sizeof(double), c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "adjoint clear");
    double4_32a *w4 = (double4_32a *)w4buf;
    const int bs = block_for(n);
    k_adj_residual<<<nblk(n, bs), bs, 0, c->stream>>>(c->a, ft, w4, acc);
    k_adj_density<<<nblk(n, bs), bs, 0, c->stream>>>(c->a, c->tab, d, ddbuf, c->cap_atoms);
    k_adj_force<<<nblk(n, bs), bs, 0, c->stream>>>(c->a, c->tab, d, w4, ddbuf, c->cap_atoms, acc);
    c->launches += 3;
    return check_launch(c, "adjoint");
}

}  // namespace msmgb
