// vv.cu -- Swope velocity Verlet on the device.
//
//   k_vv       Predictor_KERNEL0 (MD_DiffScheme_GPU.F90:242-384): DIS = h v + h^2/2 F/m,
//              x += DIS with periodic wrap, v += h/2 F/m, out-of-box flags.  In the fused
//              mode it first applies the previous step's Correction_KERNEL (:686-760),
//              v += h/2 F/m, with the same operations in the same order, so one pass over
//              x, v, F replaces the reference's two launches.  It also reduces the largest
//              displacement since the last list build (skin trigger) and refreshes the
//              float-float copy of the positions used by the list prefilter and the mixed
//              passes.
//   k_correct  Correction_KERNEL alone (end of a run, or msmgb_correction()).
//   k_decide   one thread: rebuild flag for this step from the skin trigger (or the
//              reference's fixed NB_UPTAB interval, MD_Method_GenericMD_GPU.F90:599-601).
#include "msmgb_internal.cuh"

namespace msmgb {

__device__ __forceinline__ double mi(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

__device__ __forceinline__ float mi32(float s, float len, float half, int pd)
{
    return (pd && fabsf(s) > half) ? s - copysignf(len, s) : s;
}

__device__ __forceinline__ void block_max_flush(double v, unsigned long long *dst)
{
    __shared__ double sm[kBlock / 32];
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

// order-preserving integer key of a double: x > y <=> key(x) > key(y)
__device__ __forceinline__ long long okey(double x)
{
    const long long k = __double_as_longlong(x);
    return k ^ ((k >> 63) & 0x7fffffffffffffffLL);
}

// one coordinate of Predictor_KERNEL0 (:314-349): DIS = h v + h^2/2 a (0 if FIXPOS), x += DIS,
// periodic wrap when x > lo + L or x < lo.  The box tests compare integer keys (same order
// as the doubles) so they stay off the FP64 pipe, which bounds this kernel on GB300.
__device__ __forceinline__ double advance(double x0, double v, double a, double th, double h2s2, bool fix,
                                          int pd, double len, long long klo, long long kub, double &dis,
                                          int &oob_hi, int &oob_lo)
{
    double d = fix ? 0.0 : fma(h2s2, a, th * v);
    double x = x0 + d;
    long long k = okey(x);
    if (pd) {
        if (k > kub) { x = x - len; k = okey(x); }
        else if (k < klo) { x = x + len; k = okey(x); }
    }
    oob_hi |= k > kub;
    oob_lo |= k < klo;
    dis = d;
    return x;
}

// mode 0: predictor only; mode 1: corrector of the previous step first when
// flags[kFlagPending] is set (graph replay), mode 2: always fused.
__global__ void __launch_bounds__(kBlock) k_vv(DevAtoms a, double th, int mode)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dmax = 0.0;
    const int pend = (mode == 2) ? 1 : (mode == 1 ? a.flags[kFlagPending] : 0);
    if (i < a.n) {
        int stat = a.statu[i];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const double hs2 = th * 0.5, h2s2 = th * th * 0.5;
            const DevBox &b = a.box[a.boxid[i]];
            // F/m as a product with the reciprocal mass: FP64 division is emulated and
            // costly on this GPU's FP64 pipe; the result differs from FP/CM0 by <= 1 ulp
            const double icm = a.icm[a.ityp[i] - 1];
            double4_32a p = a.pos[i];
            double vx = a.vx[i], vy = a.vy[i], vz = a.vz[i];
            const double ax = a.fx[i] * icm, ay = a.fy[i] * icm, az = a.fz[i] * icm;
            const bool fvx = (stat & (MSMGB_STATU_FIXVELX | MSMGB_STATU_FIXPOSX)) != 0;
            const bool fvy = (stat & (MSMGB_STATU_FIXVELY | MSMGB_STATU_FIXPOSY)) != 0;
            const bool fvz = (stat & (MSMGB_STATU_FIXVELZ | MSMGB_STATU_FIXPOSZ)) != 0;
            if (pend) {                 // Correction_KERNEL of the previous step
                if (!fvx) vx = fma(hs2, ax, vx);
                if (!fvy) vy = fma(hs2, ay, vy);
                if (!fvz) vz = fma(hs2, az, vz);
            }
            int hi = 0, lo = 0;
            double dx, dy, dz;
            const double x = advance(p.x, vx, ax, th, h2s2, (stat & MSMGB_STATU_FIXPOSX) != 0, b.ifpd[0],
                                     b.len[0], b.klo[0], b.kub[0], dx, hi, lo);
            const double y = advance(p.y, vy, ay, th, h2s2, (stat & MSMGB_STATU_FIXPOSY) != 0, b.ifpd[1],
                                     b.len[1], b.klo[1], b.kub[1], dy, hi, lo);
            const double z = advance(p.z, vz, az, th, h2s2, (stat & MSMGB_STATU_FIXPOSZ) != 0, b.ifpd[2],
                                     b.len[2], b.klo[2], b.kub[2], dz, hi, lo);
            if (!fvx) vx = fma(hs2, ax, vx);
            if (!fvy) vy = fma(hs2, ay, vy);
            if (!fvz) vz = fma(hs2, az, vz);
            a.pos[i] = make_double4_32a(x, y, z, p.w);
            const PosFF f = make_posff(x, y, z, b);
            a.posff[i] = f;
            a.vx[i] = vx; a.vy[i] = vy; a.vz[i] = vz;
            a.dx[i] += dx; a.dy[i] += dy; a.dz[i] += dz;
            // Predictor_KERNEL0 :372-378 (PASSBOUND is not stored, quirk Q10)
            if (hi) a.statu[i] = MSMGB_STATU_OUTOFBOX | MSMGB_STATU_REFLECT;
            else if (lo) a.statu[i] = MSMGB_STATU_OUTOFBOX | MSMGB_STATU_TRANSMIT;
            // displacement since the last build from the exact FP32 hi parts (the trigger
            // needs ~1e-4 A, the hi parts are within 3e-5 A of the FP64 positions)
            const float4 q = a.pos_bld[i];
            float ex = mi32(f.hx - q.x, b.lenf[0], b.halff[0], b.ifpd[0]);
            float ey = mi32(f.hy - q.y, b.lenf[1], b.halff[1], b.ifpd[1]);
            float ez = mi32(f.hz - q.z, b.lenf[2], b.halff[2], b.ifpd[2]);
            dmax = (double)(ex * ex + ey * ey + ez * ez);
        }
    }
    block_max_flush(dmax, a.maxdisp);
}

__global__ void __launch_bounds__(kBlock) k_correct(DevAtoms a, double th, int only_if_pending)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (only_if_pending && a.flags[kFlagPending] == 0) return;
    if (i >= a.n) return;
    int stat = a.statu[i];
    if ((stat & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) return;
    const double hs2 = th * 0.5;
    const double icm = a.icm[a.ityp[i] - 1];
    if (!(stat & MSMGB_STATU_FIXVELX) && !(stat & MSMGB_STATU_FIXPOSX)) a.vx[i] = a.vx[i] + hs2 * (a.fx[i] * icm);
    if (!(stat & MSMGB_STATU_FIXVELY) && !(stat & MSMGB_STATU_FIXPOSY)) a.vy[i] = a.vy[i] + hs2 * (a.fy[i] * icm);
    if (!(stat & MSMGB_STATU_FIXVELZ) && !(stat & MSMGB_STATU_FIXPOSZ)) a.vz[i] = a.vz[i] + hs2 * (a.fz[i] * icm);
}

__global__ void k_clear_pending(int *flags) { flags[kFlagPending] = 0; }

__global__ void k_decide(int *flags, unsigned long long *maxdisp, double thr2, int nb_uptab)
{
    int rebuild = 0;
    if (thr2 > 0.0) {
        rebuild = __longlong_as_double((long long)*maxdisp) > thr2;
    } else if (nb_uptab > 0) {
        int step = ++flags[kFlagStep];
        rebuild = (step % nb_uptab) == 0;
    }
    flags[kFlagRebuild] = rebuild;
    if (rebuild) flags[kFlagRebuilds] += 1;
    *maxdisp = 0ull;
    flags[kFlagPending] = 1;
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

int launch_vv(msmgb_ctx *c, double h, int mode)
{
    const int bs = block_for(c->n);
    k_vv<<<nblk(c->n, bs), bs, 0, c->stream>>>(c->a, h, mode);
    c->launches += 1;
    return check_launch(c, "integrator");
}

int launch_correct(msmgb_ctx *c, double h, bool only_if_pending)
{
    const int bs = block_for(c->n);
    k_correct<<<nblk(c->n, bs), bs, 0, c->stream>>>(c->a, h, only_if_pending ? 1 : 0);
    k_clear_pending<<<1, 1, 0, c->stream>>>(c->a.flags);
    c->launches += 2;
    return check_launch(c, "corrector");
}

int launch_decide(msmgb_ctx *c, double skin_trigger, int nb_uptab)
{
    double thr2 = skin_trigger > 0.0 ? skin_trigger * skin_trigger : 0.0;
    k_decide<<<1, 1, 0, c->stream>>>(c->a.flags, c->a.maxdisp, thr2, nb_uptab);
    c->launches += 1;
    return check_launch(c, "rebuild decision");
}

}  // namespace msmgb
