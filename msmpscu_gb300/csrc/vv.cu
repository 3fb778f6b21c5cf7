// vv.cu -- Swope velocity Verlet on the device.
//
//   k_vv       Predictor_KERNEL0 (MD_DiffScheme_GPU.F90:242-384): DIS = h v + h^2/2 F/m,
//              x += DIS with periodic wrap, v += h/2 F/m, out-of-box flags.  In the fused
//              mode it first applies the previous step's Correction_KERNEL (:686-760),
//              v += h/2 F/m, with the same operations in the same order, so one pass over
//              x, v, F replaces the reference's two launches.  It also reduces the largest
//              displacement since the last list build (skin trigger) and refreshes the
//              float-float copy of the positions used by the list prefilter and the mixed
//              passes.  The per-atom work is vv_atom() in msmgb_internal.cuh, shared with
//              the fused mixed force kernel.  Under the mixed-precision passes it runs the
//              form of the update with fewer FP64 instructions (vv_atom<true>) that the
//              fused mixed kernel runs, so a fused and an unfused step stay bitwise equal.
//   k_correct  Correction_KERNEL alone (end of a run, or msmgb_correction()).
//   k_decide   one thread: rebuild flag for this step from the skin trigger (or the
//              reference's fixed NB_UPTAB interval, MD_Method_GenericMD_GPU.F90:599-601);
//              in a step graph it also sets the conditional node that runs the rebuild.
//   k_set_full one thread, first node of a two-level rebuild body: sets the nested
//              conditional node of the full rebuild from the decision.
#include "msmgb_internal.cuh"

namespace msmgb {

// mode 0: predictor only; mode 1: corrector of the previous step first when
// flags[kFlagPending] is set (graph replay), mode 2: always fused.
template <bool HV>
__global__ void __launch_bounds__(kBlock) k_vv(DevAtoms a, double th, int mode)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float dmax = 0.0f;
    const int pend = (mode == 2) ? 1 : (mode == 1 ? a.flags[kFlagPending] : 0);
    if (i < a.n) {
        const int stat = a.statu[i];
        if ((stat & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
            const DevBox &b = a.box[a.boxid[i]];
            const double4_32a p = a.pos[i];
            dmax = vv_atom<HV>(a, i, stat, b, th, pend != 0, a.fx[i], a.fy[i], a.fz[i], p, a.pos, a.posff);
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

// Inside a step graph the decision also switches the graph's conditional rebuild node.
// Two-level list (half_outer > 0): a rebuild is full (binning, sort, candidates) when the
// displacement since the last full rebuild may exceed half the outer skin, bounded by the sum
// of the interval maxima (each the largest displacement since the previous build); otherwise
// only the list is re-selected from the candidates.  Single-level list: cond, the rebuild
// body.  Two-level list: cond_inner, the body that runs on every rebuild; the full rebuild is
// a conditional node nested in that body (a step without a rebuild evaluates one node), whose
// condition k_set_full sets there from flags[kFlagFullNow].
__global__ void k_decide(int *flags, unsigned long long *maxdisp, double thr2, int nb_uptab,
                         cudaGraphConditionalHandle cond, int use_cond, float half_outer,
                         cudaGraphConditionalHandle cond_inner)
{
    int rebuild = 0;
    const double md2 = __longlong_as_double((long long)*maxdisp);
    if (thr2 > 0.0) {
        rebuild = md2 > thr2;
    } else if (nb_uptab > 0) {
        int step = ++flags[kFlagStep];
        rebuild = (step % nb_uptab) == 0;
    }
    int full = rebuild;
    if (rebuild && half_outer > 0.0f) {
        const float acc = __int_as_float(flags[kFlagAcc]) + (float)sqrt(md2);
        full = !(acc <= half_outer) || flags[kFlagOob] != 0;
        flags[kFlagAcc] = __float_as_int(full ? 0.0f : acc);
        if (full) flags[kFlagFull] += 1;
    }
    flags[kFlagRebuild] = rebuild;
    if (rebuild) flags[kFlagRebuilds] += 1;
    flags[kFlagFullNow] = full;
    if (use_cond) {
        if (half_outer > 0.0f) cudaGraphSetConditional(cond_inner, rebuild ? 1u : 0u);
        else cudaGraphSetConditional(cond, full ? 1u : 0u);
    }
    *maxdisp = 0ull;
    flags[kFlagPending] = 1;
}

__global__ void k_set_full(const int *flags, cudaGraphConditionalHandle cond_full)
{
    cudaGraphSetConditional(cond_full, flags[kFlagFullNow] ? 1u : 0u);
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

int launch_vv(msmgb_ctx *c, double h, int mode)
{
    const int bs = block_for(c->n);
    if (c->p.precision == MSMGB_PREC_MIXED)
        k_vv<true><<<nblk(c->n, bs), bs, 0, c->stream>>>(c->a, h, mode);
    else
        k_vv<false><<<nblk(c->n, bs), bs, 0, c->stream>>>(c->a, h, mode);
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

int launch_set_full(msmgb_ctx *c, cudaGraphConditionalHandle cond_full)
{
    k_set_full<<<1, 1, 0, c->stream>>>(c->a.flags, cond_full);
    c->launches += 1;
    return check_launch(c, "rebuild decision");
}

int launch_decide(msmgb_ctx *c, double skin_trigger, int nb_uptab, cudaGraphConditionalHandle cond, bool use_cond,
                  cudaGraphConditionalHandle cond_inner)
{
    double thr2 = skin_trigger > 0.0 ? skin_trigger * skin_trigger : 0.0;
    // the displacement bound comes from the FP32 positions hi + lo (within 3e-5 A of the positions): 1e-3 A margin
    const float half_outer = (use_cond && two_level(c)) ? (float)(0.5 * c->outer_skin - 1e-3) : 0.0f;
    k_decide<<<1, 1, 0, c->stream>>>(c->a.flags, c->a.maxdisp, thr2, nb_uptab, cond, use_cond ? 1 : 0, half_outer,
                                     cond_inner);
    c->launches += 1;
    return check_launch(c, "rebuild decision");
}

}  // namespace msmgb
