// context.cu -- the C ABI: context, table upload, state transfer, the MD step graph.
//
// Device state lives in one context object instead of the reference's module globals
// (dm_WorkSpace, dm_FTableWS, dm_Neighbors; MD_Globle_Variables_GPU.F90:158-194).  All
// work is issued on the context's stream; the per-step sequence of For_One_Step
// (MD_Method_GenericMD_GPU.F90:596-627: Predictor_DEV, Cal_NeighBoreList_DEV every
// NB_UPTAB steps, CalForce, Correction_DEV) is captured once as a CUDA graph whose list
// rebuild sits in a conditional node that the step's decision kernel switches on the
// device, so a step costs one graph launch and no host synchronisation.  In the mixed and
// float-float modes the force pass and the integrator are one kernel and the graphs
// alternate two position buffers.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "msmgb_internal.cuh"

using namespace msmgb;

namespace msmgb {

int set_err(msmgb_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_err(msmgb_ctx *c, cudaError_t e, const char *what)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "CUDA error in %s: %s (%s)", what, cudaGetErrorName(e),
             cudaGetErrorString(e));
    return set_err(c, MSMGB_ERR_CUDA, buf);
}

int check_launch(msmgb_ctx *c, const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, what);
    return MSMGB_OK;
}

}  // namespace msmgb

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_err(c, e_, what); \
    } while (0)

#define RET(x)                      \
    do {                            \
        int r_ = (x);               \
        if (r_ != MSMGB_OK) return r_; \
    } while (0)

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

// integer key that orders like the double value (for the integrator's box tests)
static long long order_key(double x)
{
    long long k;
    memcpy(&k, &x, sizeof(k));
    return k ^ ((k >> 63) & 0x7fffffffffffffffLL);
}

template <typename T>
static cudaError_t dalloc(T **p, size_t count)
{
    return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}

static void free_graph(msmgb_ctx *c)
{
    if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
    c->step_graph = nullptr;
    c->graph_n = -1;
    cudaGraphExec_t *gs[8] = {&c->g_pre,    &c->g_loop[0],  &c->g_loop[1],  &c->g_final[0],
                              &c->g_final[1], &c->g_loopk[0], &c->g_loopk[1], &c->step_graphk};
    for (cudaGraphExec_t *g : gs) {
        if (*g) cudaGraphExecDestroy(*g);
        *g = nullptr;
    }
    c->fg_n = -1;
}

static int use_device(msmgb_ctx *c)
{
    CK(cudaSetDevice(c->p.device), "cudaSetDevice");
    return MSMGB_OK;
}

// ---- small kernels of the ABI -------------------------------------------------------------
__global__ void k_pack(DevAtoms a, const double *xp, const double *xp1, const int *ityp,
                       const int *statu, const int *boxid)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = a.n;
    if (i >= n) return;
    double x = xp[i], y = xp[n + i], z = xp[2 * n + i];
    bool fin = isfinite(x) && isfinite(y) && isfinite(z);
    if (xp1) fin = fin && isfinite(xp1[i]) && isfinite(xp1[n + i]) && isfinite(xp1[2 * n + i]);
    if (!fin) atomicOr(&a.flags[kFlagErr], kErrNonFinite);
    a.pos[i] = make_double4_32a(x, y, z, 0.0);
    PosFF f = make_posff(x, y, z, a.box[boxid[i]]);
    a.posff[i] = f;
    a.pos_bld[i] = pos_f32(f);
    a.vx[i] = xp1 ? xp1[i] : 0.0;
    a.vy[i] = xp1 ? xp1[n + i] : 0.0;
    a.vz[i] = xp1 ? xp1[2 * n + i] : 0.0;
    a.fx[i] = 0.0; a.fy[i] = 0.0; a.fz[i] = 0.0;
    a.dx[i] = 0.0; a.dy[i] = 0.0; a.dz[i] = 0.0;
    a.ityp[i] = ityp[i];
    a.statu[i] = statu[i];
    a.gid[i] = i;
    a.boxid[i] = boxid[i];
    a.den[i] = 0.0;
    a.epot[i] = 0.0;
}

// sorted -> caller layout: dst[k*n + g] = src_k[s] with g = gid[s] (or s when sorted)
__global__ void k_unpack3(const double *s0, const double *s1, const double *s2, const int *gid,
                          int n, int sorted, double *dst)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int g = sorted ? s : gid[s];
    dst[g] = s0[s];
    if (s1) dst[n + g] = s1[s];
    if (s2) dst[2 * n + g] = s2[s];
}

// caller-order positions -> sorted state (periodic directions wrapped into the box); the
// largest displacement since the last list build goes to maxdisp (skin check)
__global__ void __launch_bounds__(kBlock) k_update_pos(DevAtoms a, const double *xp)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    double d2 = 0.0;
    bool ok = false;
    double x[3] = {0.0, 0.0, 0.0};
    if (s < a.n) {
        const int n = a.n, g = a.gid[s];
        x[0] = xp[g];
        x[1] = xp[n + g];
        x[2] = xp[2 * n + g];
        ok = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
        if (!ok) atomicOr(&a.flags[kFlagErr], kErrNonFinite);   // that atom keeps its old position
    }
    if (ok) {
        const DevBox &b = a.box[a.boxid[s]];
#pragma unroll
        bool out = false;
        for (int k = 0; k < 3; ++k) {
            if (b.ifpd[k]) x[k] -= floor((x[k] - b.lo[k]) / b.len[k]) * b.len[k];
            else out |= x[k] < b.lo[k] || x[k] > b.lo[k] + b.len[k];
        }
        if (out) atomicOr(&a.flags[kFlagOob], 1);   // the next list build re-bins every atom
        a.pos[s] = make_double4_32a(x[0], x[1], x[2], 0.0);
        const PosFF f = make_posff(x[0], x[1], x[2], b);
        a.posff[s] = f;
        const float4 q = a.pos_bld[s];
        const float4 g = pos_f32(f);
        const float ex = mi32f(g.x - q.x, b.lenf[0], b.halff[0], b.ifpd[0]);
        const float ey = mi32f(g.y - q.y, b.lenf[1], b.halff[1], b.ifpd[1]);
        const float ez = mi32f(g.z - q.z, b.lenf[2], b.halff[2], b.ifpd[2]);
        d2 = (double)(ex * ex + ey * ey + ez * ez);
    }
    block_max_flush(d2, a.maxdisp);
}

// per-atom kinetic energy in the sorted order (CALEKIN_KERNEL, MD_DiffScheme_GPU.F90:851-902):
// 0.5 m v^2 for an active atom with no fixed position component, else -1e32
__global__ void k_ekin(DevAtoms a, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int st = a.statu[i];
    double ek = -1.0e32;
    if ((st & MSMGB_STATU_ACTIVE) && !(st & (MSMGB_STATU_FIXPOSX | MSMGB_STATU_FIXPOSY | MSMGB_STATU_FIXPOSZ))) {
        const double m = a.cm[a.ityp[i] - 1];
        ek = 0.5 * m * (a.vx[i] * a.vx[i] + a.vy[i] * a.vy[i] + a.vz[i] * a.vz[i]);
    }
    out[i] = ek;
}

__global__ void k_unpack_pos(const double4_32a *pos, const int *gid, int n, int sorted, double *dst)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int g = sorted ? s : gid[s];
    double4_32a p = pos[s];
    dst[g] = p.x;
    dst[n + g] = p.y;
    dst[2 * n + g] = p.z;
}

__global__ void k_f32_to_f64(const float *src, int n, double *dst)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dst[s] = (double)src[s];
}

__global__ void k_unpack_int(const int *src, const int *gid, int n, int sorted, int *dst)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    dst[sorted ? s : gid[s]] = src[s];
}

// ---- context ------------------------------------------------------------------------------
extern "C" int msmgb_create(msmgb_ctx **out, const msmgb_params *p)
{
    if (!out || !p) return MSMGB_ERR_ARG;
    *out = nullptr;
    if (p->max_atoms <= 0 || p->max_boxes <= 0 || p->mxkvois <= 0 || p->rc_nl <= 0.0)
        return MSMGB_ERR_ARG;
    if (p->precision != MSMGB_PREC_FP64 && p->precision != MSMGB_PREC_MIXED && p->precision != MSMGB_PREC_FF)
        return MSMGB_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device || p->device < 0) {
        cudaGetLastError();
        return MSMGB_ERR_NO_DEVICE;
    }
    msmgb_ctx *c = new msmgb_ctx();
    c->p = *p;
    {
        const char *chk = getenv("MSMGB_CHECK_LISTS");
        c->check_lists = chk && chk[0] == '1';
    }
    c->cap_atoms = p->max_atoms;
    c->cap_boxes = p->max_boxes;
    int rc = use_device(c);
    if (rc) { delete c; return rc; }
    auto fail = [&](cudaError_t e, const char *w) {
        cuda_err(c, e, w);
        msmgb_destroy(c);
        return MSMGB_ERR_CUDA;
    };
    cudaError_t e;
    if (p->stream) {
        c->stream = (cudaStream_t)p->stream;
    } else {
        if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
            return fail(e, "stream");
        c->own_stream = true;
    }
    const size_t N = (size_t)c->cap_atoms;
    DevAtoms &a = c->a;
    a.mxk = p->mxkvois;
    // ELL leading dimension: a multiple of 256 atoms, so a block's tile of the list (256 atoms x
    // some slots) never leaves the allocation and a row is a multiple of 16 bytes (TMA)
    a.ld = (int)((((size_t)c->cap_atoms + 255) / 256) * 256);
    const size_t LD = (size_t)a.ld;
#define AL(ptr, cnt)                                            \
    if ((e = dalloc(&(ptr), (cnt))) != cudaSuccess) return fail(e, "cudaMalloc " #ptr);
    AL(a.pos, N) AL(a.posff, N) AL(a.pos_bld, N)
    AL(a.vx, N) AL(a.vy, N) AL(a.vz, N)
    AL(a.fx, N) AL(a.fy, N) AL(a.fz, N)
    AL(a.dx, N) AL(a.dy, N) AL(a.dz, N)
    AL(a.ityp, N) AL(a.statu, N) AL(a.gid, N) AL(a.boxid, N)
    AL(a.den, N) AL(a.epot, N) AL(a.den32, N)
    AL(a.kvois, N) AL(a.indi, LD * (size_t)p->mxkvois)
    AL(c->cell_of, N) AL(c->perm, N)
    AL(c->dbox, (size_t)c->cap_boxes)
    AL(c->cm, (size_t)kMaxGroups)
    AL(c->icm, (size_t)kMaxGroups)
    AL(c->flags, (size_t)kFlagWords)
    AL(c->maxdisp, 1)
    AL(c->virial, 6 * (size_t)c->cap_boxes)
#undef AL
    // permutation staging: double4_32a + 6 doubles + 5 ints per atom
    if ((e = cudaMalloc(&c->scratch, N * (32 + 48 + 20) + 256)) != cudaSuccess) return fail(e, "scratch");
    if ((e = cudaMallocHost((void **)&c->h_flags, sizeof(int) * kFlagWords)) != cudaSuccess) return fail(e, "pinned");
    if ((e = cudaMallocHost((void **)&c->h_virial, sizeof(double) * 6 * c->cap_boxes)) != cudaSuccess) return fail(e, "pinned");
    if ((e = cudaMemsetAsync(c->flags, 0, sizeof(int) * kFlagWords, c->stream)) != cudaSuccess) return fail(e, "memset");
    if ((e = cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream)) != cudaSuccess) return fail(e, "memset");
    if (p->precision == MSMGB_PREC_MIXED &&
        ((e = dalloc(&a.pk, LD * (size_t)p->mxkvois)) != cudaSuccess || (e = dalloc(&a.rec16, N)) != cudaSuccess))
        return fail(e, "cudaMalloc pair index");
    if (p->precision != MSMGB_PREC_FP64 && (e = dalloc(&a.rec, N)) != cudaSuccess)
        return fail(e, "cudaMalloc records");
    if (p->precision == MSMGB_PREC_FF && ((e = dalloc(&a.posfx, N)) != cudaSuccess || (e = dalloc(&a.recfx, N)) != cudaSuccess))
        return fail(e, "cudaMalloc float-float records");
    a.flags = c->flags;
    a.maxdisp = c->maxdisp;
    a.virial = c->virial;
    a.box = c->dbox;
    a.cm = c->cm;
    a.icm = c->icm;
    a.n = 0;
    *out = c;
    return MSMGB_OK;
}

extern "C" int msmgb_destroy(msmgb_ctx *c)
{
    if (!c) return MSMGB_OK;
    cudaSetDevice(c->p.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_graph(c);
    DevAtoms &a = c->a;
    void *ptrs[] = {a.pos, a.posff, a.pos_bld, a.vx, a.vy, a.vz, a.fx, a.fy, a.fz,
                    a.dx, a.dy, a.dz, a.ityp, a.statu, a.gid, a.boxid, a.den, a.epot,
                    a.den32, a.kvois, a.indi, a.pk, a.rec, a.rec16, a.posfx, a.recfx, c->cell_of, c->perm, c->dbox, c->cm, c->icm,
                    c->flags, c->maxdisp, c->virial, c->scratch, c->cell_start,
                    c->cell_cursor, c->scan_tmp, c->cell_rank, c->cell_unrank, c->tab_mem, c->adj_mem, c->hvp_pair,
                    c->pos2, c->posff2, a.lidx, a.hmeta, a.hruns, c->cand, c->kcand, c->ext_field};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (c->h_flags) cudaFreeHost(c->h_flags);
    if (c->h_virial) cudaFreeHost(c->h_virial);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MSMGB_OK;
}

extern "C" const char *msmgb_last_error(const msmgb_ctx *c) { return c ? c->err.c_str() : "null context"; }
extern "C" void *msmgb_stream(const msmgb_ctx *c) { return c ? (void *)c->stream : nullptr; }
extern "C" int64_t msmgb_launch_count(const msmgb_ctx *c) { return c ? c->launches : 0; }

extern "C" int msmgb_set_precision(msmgb_ctx *c, int precision)
{
    if (!c) return MSMGB_ERR_ARG;
    if (precision != MSMGB_PREC_FP64 && precision != MSMGB_PREC_MIXED && precision != MSMGB_PREC_FF)
        return set_err(c, MSMGB_ERR_ARG, "precision must be MSMGB_PREC_FP64, MSMGB_PREC_MIXED or MSMGB_PREC_FF");
    if (precision == MSMGB_PREC_MIXED && !c->a.pk) {
        RET(use_device(c));
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        CK(dalloc(&c->a.pk, (size_t)c->a.ld * (size_t)c->p.mxkvois), "cudaMalloc pair index");
        CK(dalloc(&c->a.rec16, (size_t)c->cap_atoms), "cudaMalloc fixed-point records");
        bool fix_ok = !c->hbox.empty();
        for (const DevBox &b : c->hbox)
            for (int k = 0; k < 3; ++k) fix_ok = fix_ok && (b.ifpd[k] ? b.len[k] : 2.0 * b.len[k]) <= kFixMaxSpan;
        c->a.fix_on = fix_ok ? 1 : 0;
    }
    if (precision == MSMGB_PREC_FF && !c->a.posfx) {
        RET(use_device(c));
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        CK(dalloc(&c->a.posfx, (size_t)c->cap_atoms), "cudaMalloc float-float records");
        CK(dalloc(&c->a.recfx, (size_t)c->cap_atoms), "cudaMalloc float-float records");
    }
    if (precision != MSMGB_PREC_FP64 && !c->a.rec) {
        RET(use_device(c));
        CK(dalloc(&c->a.rec, (size_t)c->cap_atoms), "cudaMalloc records");
    }
    if (precision != c->p.precision) {
        c->p.precision = precision;
        c->force_valid = false;
        free_graph(c);
    }
    return MSMGB_OK;
}

extern "C" int msmgb_synchronize(msmgb_ctx *c)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(use_device(c));
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MSMGB_OK;
}

// reads the device flags; converts error bits into a status code
static int poll_flags(msmgb_ctx *c)
{
    CK(cudaMemcpyAsync(c->h_flags, c->flags, sizeof(int) * kFlagWords, cudaMemcpyDeviceToHost, c->stream),
       "flag read");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    int e = c->h_flags[kFlagErr];
    if (e) {
        CK(cudaMemsetAsync(c->flags + kFlagErr, 0, sizeof(int), c->stream), "flag clear");
        if (e & kErrOverflow) {
            char buf[160];
            snprintf(buf, sizeof(buf), "neighbour list overflow: an atom has more than MXKVOIS=%d neighbours", c->p.mxkvois);
            return set_err(c, MSMGB_ERR_NL_OVERFLOW, buf);
        }
        if (e & kErrCandOverflow) {
            c->list_valid = false;     // the next host-side build grows the candidate buffer
            char buf[200];
            snprintf(buf, sizeof(buf), "candidate list overflow: an atom has more than %d candidates within "
                     "rc_nl + outer skin (raise MXKVOIS or lower the outer skin)", c->mxo);
            return set_err(c, MSMGB_ERR_NL_OVERFLOW, buf);
        }
        if (e & kErrOutOfBox) return set_err(c, MSMGB_ERR_OUT_OF_BOX, "an active atom lies outside its box");
        if (e & kErrRho) return set_err(c, MSMGB_ERR_RHO_RANGE, "electron density beyond the F(rho) table");
        if (e & kErrTimeout)
            return set_err(c, MSMGB_ERR_TIMEOUT, "a bounded wait for an asynchronous list copy ran out");
        if (e & kErrNonFinite) return set_err(c, MSMGB_ERR_ARG, "a position is not a finite number");
        if (e & kErrBadList) return set_err(c, MSMGB_ERR_CUDA, "neighbour list validation failed");
    }
    return MSMGB_OK;
}

// a state with a non-cubic box supports the FP64 static calls only
static int need_cubic(msmgb_ctx *c, const char *what)
{
    if (!c->any_shaped) return MSMGB_OK;
    return set_err(c, MSMGB_ERR_ARG, std::string(what) + " needs cubic boxes (a BOXSHAPE is set; the FP64 "
                                                         "force, energy, virial and stress calls support it)");
}

// ---- force table ----------------------------------------------------------------------------
extern "C" int msmgb_init_forcetable(msmgb_ctx *c, const msmgb_forcetable *ft)
{
    NvtxRange nvtx_range("msmgb_init_forcetable");
    if (!c || !ft) return MSMGB_ERR_ARG;
    if (ft->pottype != MSMGB_FS_TYPE && ft->pottype != MSMGB_EAM_TYPE)
        return set_err(c, MSMGB_ERR_ARG, "unknown potential type");
    if (ft->ntab < 2 || ft->nkind < 1 || ft->rmax <= 0.0 || !ft->potr || !ft->fpotr || !ft->potb || !ft->fpotb)
        return set_err(c, MSMGB_ERR_ARG, "incomplete pair tables");
    if (ft->ngroup < 1 || ft->ngroup > kMaxGroups || !ft->kpair)
        return set_err(c, MSMGB_ERR_ARG, "NGROUP must be 1..16 with KPAIR given");
    const bool eam = ft->pottype == MSMGB_EAM_TYPE;
    if (eam && (ft->nembd < 2 || ft->nkind1 < 1 || !ft->fembd || !ft->dfembd || !ft->kembd || ft->rhod <= 0.0))
        return set_err(c, MSMGB_ERR_ARG, "EAM tables need FEMBD, DFEMBD, KEMBD and RHOD");
    RET(use_device(c));
    DevTables t{};
    t.pottype = ft->pottype;
    t.ntab = ft->ntab;
    t.nkind = ft->nkind;
    t.ntp = ft->ntab + 2;
    t.csi = (double)ft->ntab / std::sqrt(ft->rmax);
    t.ru2 = ft->ru * ft->ru;
    t.ngroup = ft->ngroup;
    for (int i = 0; i < ft->ngroup; ++i)
        for (int j = 0; j < ft->ngroup; ++j) {
            int id = ft->kpair[j * ft->ngroup + i];      // KPAIR(i,j), column-major
            if (id < 1 || id > ft->nkind) return set_err(c, MSMGB_ERR_ARG, "KPAIR id out of range");
            t.kpair[j * ft->ngroup + i] = id - 1;
        }
    t.nembd = eam ? ft->nembd : 0;
    t.nkind1 = eam ? ft->nkind1 : 0;
    t.nep = eam ? ft->nembd + 2 : 0;
    t.rhod = eam ? ft->rhod : 1.0;
    if (eam)
        for (int i = 0; i < ft->ngroup; ++i) {
            int id = ft->kembd[i];
            if (id < 1 || id > ft->nkind1) return set_err(c, MSMGB_ERR_ARG, "KEMBD id out of range");
            t.kembd[i] = id - 1;
        }
    // padded rows: index 0 -> 0, 1..NTAB -> table, NTAB+1 -> T(NTAB) (read with DK = 0 when r = Rmax)
    const size_t rowp = (size_t)t.ntp, nk = (size_t)t.nkind, nk1 = (size_t)t.nkind1, nep = (size_t)t.nep;
    const size_t nd = 4 * nk * rowp + (eam ? 2 * nk1 * nep : 0);
    std::vector<double> hd(nd, 0.0);
    const double *src[4] = {ft->potr, ft->fpotr, ft->potb, ft->fpotb};
    for (int q = 0; q < 4; ++q)
        for (size_t k = 0; k < nk; ++k) {
            double *row = hd.data() + ((size_t)q * nk + k) * rowp;
            for (int i = 1; i <= t.ntab; ++i) row[i] = src[q][(size_t)(i - 1) * nk + k];
            row[t.ntab + 1] = row[t.ntab];
        }
    if (eam) {
        const double *es[2] = {ft->fembd, ft->dfembd};
        for (int q = 0; q < 2; ++q)
            for (size_t k = 0; k < nk1; ++k) {
                double *row = hd.data() + 4 * nk * rowp + ((size_t)q * nk1 + k) * nep;
                for (int i = 1; i <= t.nembd; ++i) row[i] = es[q][(size_t)(i - 1) * nk1 + k];
                row[t.nembd + 1] = row[t.nembd];
            }
    }
    // FP32 interleaved tables of the mixed passes: value and slope (slope taken in FP64)
    const double *hpotr = hd.data(), *hfpotr = hpotr + nk * rowp, *hpotb = hpotr + 2 * nk * rowp,
                 *hfpotb = hpotr + 3 * nk * rowp;
    std::vector<float> f2((size_t)2 * nk * rowp), f4((size_t)4 * nk * rowp), e2((size_t)2 * nk1 * nep);
    for (size_t k = 0; k < nk; ++k)
        for (size_t i = 0; i < rowp; ++i) {
            size_t o = k * rowp + i, o1 = i + 1 < rowp ? o + 1 : o;
            f2[2 * o] = (float)hpotb[o];
            f2[2 * o + 1] = (float)(hpotb[o1] - hpotb[o]);
            f4[4 * o] = (float)hfpotr[o];
            f4[4 * o + 1] = (float)(hfpotr[o1] - hfpotr[o]);
            f4[4 * o + 2] = (float)hfpotb[o];
            f4[4 * o + 3] = (float)(hfpotb[o1] - hfpotb[o]);
        }
    if (eam) {
        const double *hdf = hpotr + 4 * nk * rowp + nk1 * nep;
        for (size_t k = 0; k < nk1; ++k)
            for (size_t i = 0; i < nep; ++i) {
                size_t o = k * nep + i, o1 = i + 1 < nep ? o + 1 : o;
                e2[2 * o] = (float)hdf[o];
                e2[2 * o + 1] = (float)(hdf[o1] - hdf[o]);
            }
    }
    // float-float tables: value and FP64 slope, each split into hi + lo
    auto split = [](double v, float *o) {
        o[0] = (float)v;
        o[1] = (float)(v - (double)o[0]);
    };
    std::vector<float> fd((size_t)4 * nk * rowp), ff8((size_t)8 * nk * rowp), fe((size_t)4 * nk1 * nep);
    // rows of the table-assisted mixed density pass: value, slope, r2 of the grid point
    std::vector<float> fq((size_t)4 * nk * rowp);
    for (size_t k = 0; k < nk; ++k)
        for (size_t i = 0; i < rowp; ++i) {
            size_t o = k * rowp + i;
            fq[4 * o] = f2[2 * o];
            fq[4 * o + 1] = f2[2 * o + 1];
            const double g = (double)i / t.csi, r2g = (g * g) * (g * g);
            split(r2g, &fq[4 * o + 2]);
        }
    for (size_t k = 0; k < nk; ++k)
        for (size_t i = 0; i < rowp; ++i) {
            size_t o = k * rowp + i, o1 = i + 1 < rowp ? o + 1 : o;
            split(hpotb[o], &fd[4 * o]);
            split(hpotb[o1] - hpotb[o], &fd[4 * o + 2]);
            split(hfpotr[o], &ff8[8 * o]);
            split(hfpotr[o1] - hfpotr[o], &ff8[8 * o + 2]);
            split(hfpotb[o], &ff8[8 * o + 4]);
            split(hfpotb[o1] - hfpotb[o], &ff8[8 * o + 6]);
        }
    if (eam) {
        const double *hdf = hpotr + 4 * nk * rowp + nk1 * nep;
        for (size_t k = 0; k < nk1; ++k)
            for (size_t i = 0; i < nep; ++i) {
                size_t o = k * nep + i, o1 = i + 1 < nep ? o + 1 : o;
                split(hdf[o], &fe[4 * o]);
                split(hdf[o1] - hdf[o], &fe[4 * o + 2]);
            }
    }
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (c->tab_mem) { cudaFree(c->tab_mem); c->tab_mem = nullptr; }
    const size_t bytes = nd * sizeof(double) +
                         (f2.size() + f4.size() + e2.size() + fd.size() + ff8.size() + fe.size() + fq.size()) *
                             sizeof(float) +
                         2048;
    CK(cudaMalloc(&c->tab_mem, bytes), "table alloc");
    char *base = (char *)c->tab_mem;
    double *dd = (double *)base;
    float *df4 = (float *)(base + ((nd * sizeof(double) + 255) / 256) * 256);
    float *df2 = df4 + f4.size();
    float *de2 = df2 + f2.size();
    // float4 rows: 16-byte aligned offsets
    const uintptr_t a16 = ((uintptr_t)(de2 + e2.size()) + 15) & ~(uintptr_t)15;
    float *dfd = (float *)a16;
    float *dff8 = dfd + fd.size();
    float *dfe = dff8 + ff8.size();
    float *dfq = dfe + fe.size();          // fe.size() is a multiple of 4: 16-byte aligned
    CK(cudaMemcpy(dd, hd.data(), nd * sizeof(double), cudaMemcpyHostToDevice), "table upload");
    CK(cudaMemcpy(dfd, fd.data(), fd.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    CK(cudaMemcpy(dff8, ff8.data(), ff8.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    if (eam) CK(cudaMemcpy(dfe, fe.data(), fe.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    CK(cudaMemcpy(dfq, fq.data(), fq.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    CK(cudaMemcpy(df4, f4.data(), f4.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    CK(cudaMemcpy(df2, f2.data(), f2.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    if (eam) CK(cudaMemcpy(de2, e2.data(), e2.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    t.potr = dd; t.fpotr = dd + nk * rowp; t.potb = dd + 2 * nk * rowp; t.fpotb = dd + 3 * nk * rowp;
    if (eam) {
        t.fembd = dd + 4 * nk * rowp;
        t.dfembd = t.fembd + nk1 * nep;
    }
    t.force4 = (const float4 *)df4;
    t.dens2 = (const float2 *)df2;
    t.embd2 = eam ? (const float2 *)de2 : nullptr;
    t.densff = (const float4 *)dfd;
    t.forceff = (const float4 *)dff8;
    t.embff = eam ? (const float4 *)dfe : nullptr;
    t.densq = (const float4 *)dfq;
    {
        const double ir = 1.0 / t.rhod;
        t.irhodh = (float)ir;
        t.irhodl = (float)(ir - (double)t.irhodh);
    }
    t.csih = (float)t.csi;
    t.csil = (float)(t.csi - (double)t.csih);
    t.ru2h = (float)t.ru2;
    t.ru2l = (float)(t.ru2 - (double)t.ru2h);
    t.rhodf = (float)t.rhod;
    c->tab = t;
    c->tab_rmax = ft->rmax;
    c->have_tables = true;
    c->force_valid = false;
    c->tuned_n = c->tuned_fused_n = -1;   // kernel variants are tuned per table kind count
    free_graph(c);
    return MSMGB_OK;
}

extern "C" int msmgb_clear_forcetable(msmgb_ctx *c)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(use_device(c));
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (c->tab_mem) cudaFree(c->tab_mem);
    c->tab_mem = nullptr;
    c->have_tables = false;
    c->force_valid = false;
    free_graph(c);
    return MSMGB_OK;
}

// ---- state ------------------------------------------------------------------------------------
extern "C" int msmgb_copyin_simbox(msmgb_ctx *c, int nbox, const msmgb_box *boxes, const int *ityp,
                                   const int *statu, const double *xp, const double *xp1)
{
    NvtxRange nvtx_range("msmgb_copyin_simbox");
    if (!c || !boxes || !ityp || !statu || !xp || nbox < 1) return MSMGB_ERR_ARG;
    if (nbox > c->cap_boxes) return set_err(c, MSMGB_ERR_CAPACITY, "more boxes than max_boxes");
    long total = 0;
    for (int b = 0; b < nbox; ++b) {
        if (boxes[b].natom < 0) return set_err(c, MSMGB_ERR_ARG, "negative atom count");
        total += boxes[b].natom;
    }
    if (total > c->cap_atoms) return set_err(c, MSMGB_ERR_CAPACITY, "more atoms than max_atoms");
    if (total < 1) return set_err(c, MSMGB_ERR_ARG, "no atoms");
    RET(use_device(c));
    const int n = (int)total;
    std::vector<DevBox> hb((size_t)nbox);
    const double bin_rc = c->p.rc_nl + (c->outer_skin > 0.0 ? c->outer_skin : 0.0);
    std::vector<int> boxid((size_t)n);
    int cells = 0, atom0 = 0;
    bool any_shaped = false;
    bool fix_ok = true;           // every box edge within the fixed-point records' span
    // quantum of the hi parts of the mixed positions, one power of two for all boxes: every
    // shifted coordinate u = x - lo + L in [L, 2L] (and an atom that left the box by up to L)
    // lies below 2^22 q, so that hi + 1.5 2^23 q rounds to a multiple of q, and q >= 2^-7 A
    // keeps the exact FP32 sums of squared hi differences of the density pass for pairs up to
    // ~18 A
    double posq = ldexp(1.0, -7);
    for (int b = 0; b < nbox; ++b)
        for (int k = 0; k < 3; ++k)
            if (boxes[b].len[k] > 0.0)
                posq = std::max(posq, ldexp(1.0, (int)std::ceil(std::log2(3.0 * boxes[b].len[k] / ldexp(1.0, 22)))));
    for (int b = 0; b < nbox; ++b) {
        DevBox &d = hb[(size_t)b];
        memset(&d, 0, sizeof(d));
        // BOXSHAPE (identity unless msmgb_set_boxshape gave one): a stencil cell must span
        // rc_nl after the shape, i.e. rc_nl * |row k of BOXSHAPE^-1| along box direction k
        double nrm[3] = {1.0, 1.0, 1.0};
        {
            double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            if ((size_t)(b + 1) * 9 <= c->shapes.size()) memcpy(m, &c->shapes[(size_t)b * 9], sizeof(m));
            memcpy(d.bs, m, sizeof(m));
            d.shaped = 0;
            for (int q = 0; q < 9; ++q)
                if (m[q] != ((q % 4 == 0) ? 1.0 : 0.0)) d.shaped = 1;
            if (d.shaped) {
                const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                                   m[2] * (m[3] * m[7] - m[4] * m[6]);
                if (!(fabs(det) > 1e-12)) return set_err(c, MSMGB_ERR_ARG, "BOXSHAPE is singular");
                const double inv[9] = {(m[4] * m[8] - m[5] * m[7]) / det, (m[2] * m[7] - m[1] * m[8]) / det,
                                       (m[1] * m[5] - m[2] * m[4]) / det, (m[5] * m[6] - m[3] * m[8]) / det,
                                       (m[0] * m[8] - m[2] * m[6]) / det, (m[2] * m[3] - m[0] * m[5]) / det,
                                       (m[3] * m[7] - m[4] * m[6]) / det, (m[1] * m[6] - m[0] * m[7]) / det,
                                       (m[0] * m[4] - m[1] * m[3]) / det};
                for (int k = 0; k < 3; ++k)
                    nrm[k] = sqrt(inv[3 * k] * inv[3 * k] + inv[3 * k + 1] * inv[3 * k + 1] +
                                  inv[3 * k + 2] * inv[3 * k + 2]);
                any_shaped = true;
            }
        }
        for (int k = 0; k < 3; ++k) {
            d.lo[k] = boxes[b].lo[k];
            d.len[k] = boxes[b].len[k];
            d.half[k] = 0.5 * boxes[b].len[k];
            d.ushift[k] = boxes[b].len[k] - boxes[b].lo[k];
            d.klo[k] = order_key(boxes[b].lo[k]);
            d.kub[k] = order_key(boxes[b].lo[k] + boxes[b].len[k]);
            d.lenf[k] = (float)d.len[k];
            d.lenlo[k] = (float)(d.len[k] - (double)d.lenf[k]);
            d.halff[k] = (float)d.half[k];
            d.ifpd[k] = boxes[b].ifpd[k] ? 1 : 0;
            {   // fixed-point unit: the edge (periodic) or twice the edge (open) over 2^32
                const double span = d.ifpd[k] ? d.len[k] : 2.0 * d.len[k];
                const double S = 4294967296.0 / span;
                d.fixu[k] = (float)(span / 4294967296.0);
                d.fixs[k] = (float)S;
                d.fixlq[k] = (float)(std::nearbyint(d.len[k] / posq) * posq);
                d.fixll[k] = (float)(d.len[k] - (double)d.fixlq[k]);
                d.fixa[k] = span > kFixMaxSpan ? 0ull : (unsigned long long)std::llround(posq * S * 4294967296.0);
                if (span > kFixMaxSpan) fix_ok = false;
            }
            if (d.len[k] <= 0.0) return set_err(c, MSMGB_ERR_ARG, "box length must be positive");
            // a pair within rc_nl has |SEP_k| <= rc_nl * |row k of BOXSHAPE^-1| (nrm = 1 for a
            // cubic box): the single-shift minimum image is unique only below half the edge
            if (d.ifpd[k] && d.len[k] <= 2.0 * c->p.rc_nl * nrm[k])
                return set_err(c, MSMGB_ERR_BOX_TOO_SMALL,
                               d.shaped ? "periodic box edge must exceed twice the list cutoff times the norm of "
                                          "the matching row of BOXSHAPE^-1"
                                        : "periodic box edge must exceed twice the list cutoff");
            // MD_NeighborsList_GPU.F90:289-292 with the cell size rc_nl, or rc_nl + the outer
            // skin for a two-level list (the candidates must lie in the 27-cell stencil)
            const double ncd = d.len[k] / ((d.shaped ? c->p.rc_nl : bin_rc) * nrm[k]) - 0.0001;
            if (!(ncd < (double)(1 << 24)))      // a strongly stretching BOXSHAPE
                return set_err(c, MSMGB_ERR_CAPACITY, "too many cells along one box edge");
            const int nc = (int)ncd;
            d.nc[k] = nc < 3 ? 3 : nc;
        }
        {   // hi parts are multiples of the quantum posq; |lo_i - lo_j| <= posq
            double ext = 2.0 * std::max(d.len[0], std::max(d.len[1], d.len[2]));
            d.qq = (float)posq;
            d.qinv = (float)(1.0 / posq);
            d.qmag = (float)(1.5 * ldexp(posq, 23));
            // the float-float records' fixed-point frame: 2^32 units per quantum
            d.pscale = 4294967296.0 / posq;
            d.plo = (float)(posq / 4294967296.0);
            for (int k = 0; k < 3; ++k) d.ushs[k] = d.ushift[k] * d.pscale;
            d.dlmax = (float)(2.0 * posq);
            d.dlfx = (float)(2.0 * ldexp(1.0, ilogb(ext) - 23));   // |u - float(u)| <= ulp(2L)/2
            // float-float passes: remainders u - float(u) (|.| <= ulp(2L)/2) in units of
            // 2^-30 ulp(2L), i.e. |q| <= 2^29
            const double ulp2l = ldexp(1.0, ilogb(ext) - 23);
            d.fxq = (float)ldexp(ulp2l, -30);
            d.fxinv = ldexp(1.0, 30) / ulp2l;
            for (int k = 0; k < 3; ++k) d.lq[k] = (int)llrint((d.len[k] - (double)d.lenf[k]) * d.fxinv);
        }
        long nb = (long)d.nc[0] * d.nc[1] * d.nc[2];
        if ((long)cells + nb > (1L << 24) - 2) return set_err(c, MSMGB_ERR_CAPACITY, "too many cells");
        d.cell0 = cells;
        cells += (int)nb;
        d.atom0 = atom0;
        d.natom = boxes[b].natom;
        for (int i = 0; i < boxes[b].natom; ++i) boxid[(size_t)(atom0 + i)] = b;
        atom0 += boxes[b].natom;
    }
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    {   // the step graphs hold the atom count, the cell grid and the prefilter band of the
        // box extents: a state of the same layout keeps them
        std::vector<double> gl = {(double)n, (double)nbox, bin_rc, (double)cells};
        for (int b = 0; b < nbox; ++b) {
            gl.push_back((double)boxes[b].natom);
            for (int q = 0; q < 9; ++q) gl.push_back(hb[(size_t)b].bs[q]);
            for (int k = 0; k < 3; ++k) {
                gl.push_back(boxes[b].lo[k]);
                gl.push_back(boxes[b].len[k]);
                gl.push_back((double)boxes[b].ifpd[k]);
            }
        }
        if (gl != c->graph_layout || cells + 2 > c->cap_cells) {
            free_graph(c);
            c->graph_layout = gl;
        }
    }
    if (cells + 2 > c->cap_cells) {
        if (c->cell_start) cudaFree(c->cell_start);
        if (c->cell_cursor) cudaFree(c->cell_cursor);
        if (c->scan_tmp) cudaFree(c->scan_tmp);
        if (c->cell_rank) cudaFree(c->cell_rank);
        if (c->cell_unrank) cudaFree(c->cell_unrank);
        c->cell_start = c->cell_cursor = c->scan_tmp = c->cell_rank = c->cell_unrank = nullptr;
        int cap = cells + 2;
        CK(dalloc(&c->cell_start, (size_t)cap + 1), "cell alloc");
        CK(dalloc(&c->cell_cursor, (size_t)cap + 1), "cell alloc");
        CK(dalloc(&c->scan_tmp, (size_t)(cap / 4096 + 2) + 4096), "cell alloc");
        CK(dalloc(&c->cell_rank, (size_t)cap + 1), "cell alloc");
        CK(dalloc(&c->cell_unrank, (size_t)cap + 1), "cell alloc");
        c->cap_cells = cap;
        c->rank_layout.clear();
    }
    std::vector<int> layout;
    {
        const char *env = getenv("MSMGB_CELL_ORDER");
        c->cell_row_order = env && strcmp(env, "row") == 0;
        layout.push_back(c->cell_row_order ? 1 : 0);
        for (int b = 0; b < nbox; ++b)
            for (int k = 0; k < 3; ++k) layout.push_back(hb[(size_t)b].nc[k]);
    }
    if (layout != c->rank_layout) {   // storage order of the cells: per box, Morton order of
        // (ix, iy, iz), so that atoms consecutive in memory (a warp, a CTA) occupy a compact
        // brick of cells and their neighbour records overlap; the sentinel cell of out-of-box
        // atoms stays last.  Made once per cell-grid layout.
        std::vector<int> rank((size_t)cells + 1);
        std::vector<std::pair<unsigned long long, int>> key;
        for (int b = 0; b < nbox; ++b) {
            const DevBox &d = hb[(size_t)b];
            const int nb = d.nc[0] * d.nc[1] * d.nc[2];
            key.resize((size_t)nb);
            for (int l = 0; l < nb; ++l) {
                const unsigned x = (unsigned)(l % d.nc[0]), y = (unsigned)((l / d.nc[0]) % d.nc[1]),
                               z = (unsigned)(l / (d.nc[0] * d.nc[1]));
                unsigned long long m = 0;
                for (int bit = 0; bit < 21; ++bit)
                    m |= ((unsigned long long)((x >> bit) & 1u) << (3 * bit)) |
                         ((unsigned long long)((y >> bit) & 1u) << (3 * bit + 1)) |
                         ((unsigned long long)((z >> bit) & 1u) << (3 * bit + 2));
                key[(size_t)l] = std::make_pair(c->cell_row_order ? (unsigned long long)l : m, l);
            }
            std::sort(key.begin(), key.end());
            for (int q = 0; q < nb; ++q) rank[(size_t)(d.cell0 + key[(size_t)q].second)] = d.cell0 + q;
        }
        rank[(size_t)cells] = cells;
        std::vector<int> unrank((size_t)cells + 1);
        for (int g = 0; g <= cells; ++g) unrank[(size_t)rank[(size_t)g]] = g;
        CK(cudaMemcpy(c->cell_rank, rank.data(), sizeof(int) * ((size_t)cells + 1), cudaMemcpyHostToDevice),
           "cell order upload");
        CK(cudaMemcpy(c->cell_unrank, unrank.data(), sizeof(int) * ((size_t)cells + 1), cudaMemcpyHostToDevice),
           "cell order upload");
        c->rank_layout = layout;
    }
    c->ncell_total = cells;
    c->bin_rc = bin_rc;
    c->any_shaped = any_shaped;
    c->a.fix_on = (fix_ok && c->a.rec16) ? 1 : 0;
    c->max_density = 0.0;
    for (int b = 0; b < nbox; ++b)
        c->max_density = std::max(c->max_density, boxes[b].natom / (boxes[b].len[0] * boxes[b].len[1] * boxes[b].len[2]));
    c->nbox = nbox;
    if (c->ext_field && c->ext_field_n != n) {     // the field belonged to another atom count
        cudaFree(c->ext_field);
        c->ext_field = nullptr;
        c->ext_field_n = 0;
        free_graph(c);
    }
    c->n = n;
    c->a.n = n;
    c->boxes.assign(boxes, boxes + nbox);
    c->hbox = hb;
    CK(cudaMemcpy(c->dbox, hb.data(), sizeof(DevBox) * (size_t)nbox, cudaMemcpyHostToDevice), "box upload");

    // stage the caller's arrays in the scratch buffer, then pack on the device
    char *s = (char *)c->scratch;
    double *dxp = (double *)s;
    double *dxp1 = dxp + 3 * (size_t)n;
    int *dty = (int *)(dxp1 + 3 * (size_t)n);
    int *dst = dty + n;
    int *dbx = dst + n;
    CK(cudaMemcpy(dxp, xp, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice), "copyin");
    if (xp1) CK(cudaMemcpy(dxp1, xp1, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice), "copyin");
    CK(cudaMemcpy(dty, ityp, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice), "copyin");
    CK(cudaMemcpy(dst, statu, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice), "copyin");
    CK(cudaMemcpy(dbx, boxid.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice), "copyin");
    CK(cudaMemsetAsync(c->flags, 0, sizeof(int) * kFlagWords, c->stream), "flag clear");
    k_pack<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a, dxp, xp1 ? dxp1 : nullptr, dty, dst, dbx);
    c->launches += 1;
    RET(check_launch(c, "pack"));
    {   // a non-finite position or velocity leaves the context without a state
        const int rc = poll_flags(c);
        if (rc != MSMGB_OK) {
            c->n = 0;
            c->a.n = 0;
            return rc;
        }
    }
    CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    c->list_valid = false;
    c->force_valid = false;
    return MSMGB_OK;
}

extern "C" int msmgb_set_masses(msmgb_ctx *c, int ngroup, const double *cm)
{
    if (!c || !cm || ngroup < 1 || ngroup > kMaxGroups) return MSMGB_ERR_ARG;
    for (int i = 0; i < ngroup; ++i)
        if (!(cm[i] > 0.0)) return set_err(c, MSMGB_ERR_ARG, "masses must be positive");
    RET(use_device(c));
    CK(cudaMemcpy(c->cm, cm, sizeof(double) * (size_t)ngroup, cudaMemcpyHostToDevice), "mass upload");
    double inv[kMaxGroups];
    for (int i = 0; i < ngroup; ++i) inv[i] = 1.0 / cm[i];
    CK(cudaMemcpy(c->icm, inv, sizeof(double) * (size_t)ngroup, cudaMemcpyHostToDevice), "mass upload");
    c->have_masses = true;
    return MSMGB_OK;
}

static int need_state(msmgb_ctx *c)
{
    if (c->n <= 0) return set_err(c, MSMGB_ERR_ARG, "no state: call msmgb_copyin_simbox first");
    return MSMGB_OK;
}

static int copy_out_doubles(msmgb_ctx *c, const double *s0, const double *s1, const double *s2,
                            double *host, int order)
{
    const int n = c->n;
    double *tmp = (double *)c->scratch;
    k_unpack3<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(s0, s1, s2, c->a.gid, n,
                                                       order == MSMGB_ORDER_SORTED, tmp);
    c->launches += 1;
    RET(check_launch(c, "copy-out"));
    int m = s1 ? 3 : 1;
    CK(cudaMemcpyAsync(host, tmp, sizeof(double) * (size_t)m * n, cudaMemcpyDefault, c->stream), "copy-out");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MSMGB_OK;
}

extern "C" int msmgb_copyout_simbox(msmgb_ctx *c, double *xp, double *xp1, int *statu, double *dis,
                                    int order)
{
    NvtxRange nvtx_range("msmgb_copyout_simbox");
    if (!c) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    const int n = c->n;
    const int sorted = order == MSMGB_ORDER_SORTED;
    if (xp) {
        double *tmp = (double *)c->scratch;
        k_unpack_pos<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a.pos, c->a.gid, n, sorted, tmp);
        c->launches += 1;
        RET(check_launch(c, "copy-out"));
        CK(cudaMemcpyAsync(xp, tmp, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, c->stream), "copy-out");
        CK(cudaStreamSynchronize(c->stream), "synchronize");
    }
    if (xp1) RET(copy_out_doubles(c, c->a.vx, c->a.vy, c->a.vz, xp1, order));
    if (dis) RET(copy_out_doubles(c, c->a.dx, c->a.dy, c->a.dz, dis, order));
    if (statu) {
        int *tmp = (int *)c->scratch;
        k_unpack_int<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a.statu, c->a.gid, n, sorted, tmp);
        c->launches += 1;
        RET(check_launch(c, "copy-out"));
        CK(cudaMemcpyAsync(statu, tmp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream), "copy-out");
        CK(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return MSMGB_OK;
}

extern "C" int msmgb_update_positions(msmgb_ctx *c, const double *xp)
{
    NvtxRange nvtx_range("msmgb_update_positions");
    if (!c || !xp) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    const int n = c->n;
    double *tmp = (double *)c->scratch;
    CK(cudaMemcpyAsync(tmp, xp, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, c->stream), "position copy-in");
    CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
    k_update_pos<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(c->a, tmp);
    c->launches += 1;
    RET(check_launch(c, "position update"));
    unsigned long long md = 0;
    CK(cudaMemcpyAsync(&md, c->maxdisp, sizeof(md), cudaMemcpyDeviceToHost, c->stream), "flag read");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    RET(poll_flags(c));
    double d2;
    memcpy(&d2, &md, sizeof(d2));
    const double thr = c->p.skin_trigger > 0.0 ? c->p.skin_trigger : 0.0;
    if (!(d2 <= thr * thr)) c->list_valid = false;   // moved beyond the skin: rebuild at the next call
    if (c->any_shaped) c->list_valid = false;         // the skin test is in box units: always rebuild
    CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
    c->force_valid = false;
    return MSMGB_OK;
}

// ---- several MD steps per graph launch ---------------------------------------------------------
extern "C" int msmgb_set_steps_per_graph(msmgb_ctx *c, int k)
{
    if (!c || k < 1 || k > 64) return MSMGB_ERR_ARG;
    if (k != c->steps_per_graph) {
        c->steps_per_graph = k;
        free_graph(c);
    }
    return MSMGB_OK;
}

extern "C" int msmgb_graph_launch_count(const msmgb_ctx *c, int64_t *n)
{
    if (!c || !n) return MSMGB_ERR_ARG;
    *n = c->graph_launches;
    return MSMGB_OK;
}

// ---- external forces ----------------------------------------------------------------------
extern "C" int msmgb_add_extforce(msmgb_ctx *c, const char *tag, msmgb_extforce_fn fn, void *user)
{
    if (!c || !fn) return MSMGB_ERR_ARG;
    c->ext.push_back({tag ? std::string(tag) : std::string(), fn, user});
    free_graph(c);                 // the step graphs are rebuilt, unfused, with the routine
    c->force_valid = false;
    return MSMGB_OK;
}

extern "C" int msmgb_clear_extforce(msmgb_ctx *c)
{
    if (!c) return MSMGB_ERR_ARG;
    c->ext.clear();
    if (c->ext_field) {
        RET(use_device(c));
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        cudaFree(c->ext_field);
        c->ext_field = nullptr;
    }
    c->ext_field_n = 0;
    free_graph(c);
    c->force_valid = false;
    return MSMGB_OK;
}

extern "C" int msmgb_set_extforce_field(msmgb_ctx *c, const double *fext)
{
    NvtxRange nvtx_range("msmgb_set_extforce_field");
    if (!c) return MSMGB_ERR_ARG;
    RET(use_device(c));
    if (!fext) {
        if (c->ext_field) {
            CK(cudaStreamSynchronize(c->stream), "synchronize");
            cudaFree(c->ext_field);
            c->ext_field = nullptr;
        }
        c->ext_field_n = 0;
    } else {
        RET(need_state(c));
        if (!c->ext_field) {
            CK(cudaStreamSynchronize(c->stream), "synchronize");
            CK(cudaMalloc(&c->ext_field, sizeof(double) * 3 * (size_t)c->cap_atoms), "cudaMalloc external field");
        }
        CK(cudaMemcpyAsync(c->ext_field, fext, sizeof(double) * 3 * (size_t)c->n, cudaMemcpyDefault, c->stream),
           "external field copy-in");
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        c->ext_field_n = c->n;
    }
    free_graph(c);
    c->force_valid = false;
    return MSMGB_OK;
}

extern "C" int msmgb_copyout_force(msmgb_ctx *c, double *fp, int order)
{
    NvtxRange nvtx_range("msmgb_copyout_force");
    if (!c || !fp) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    if (!c->force_valid) return set_err(c, MSMGB_ERR_ARG, "forces are not current: call msmgb_calforce");
    return copy_out_doubles(c, c->a.fx, c->a.fy, c->a.fz, fp, order);
}

extern "C" int msmgb_copyout_epot(msmgb_ctx *c, double *epot, int order)
{
    if (!c || !epot) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    return copy_out_doubles(c, c->a.epot, nullptr, nullptr, epot, order);
}

extern "C" int msmgb_calekin(msmgb_ctx *c, double *ekin, int order)
{
    NvtxRange nvtx_range("msmgb_calekin");
    if (!c || !ekin) return MSMGB_ERR_ARG;
    RET(need_state(c));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    RET(use_device(c));
    double *tmp = (double *)c->scratch + 3 * (size_t)c->cap_atoms;   // past copy_out's staging
    k_ekin<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a, tmp);
    c->launches += 1;
    RET(check_launch(c, "kinetic energy"));
    return copy_out_doubles(c, tmp, nullptr, nullptr, ekin, order);
}

extern "C" int msmgb_copyout_den(msmgb_ctx *c, double *den, int order)
{
    if (!c || !den) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    if (c->den_is32) {   // the last density pass was the mixed one: F'(rho) is held in FP32
        double *conv = (double *)((char *)c->scratch + 64 * (size_t)c->cap_atoms);
        k_f32_to_f64<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a.den32, c->n, conv);
        c->launches += 1;
        RET(check_launch(c, "copy-out"));
        return copy_out_doubles(c, conv, nullptr, nullptr, den, order);
    }
    return copy_out_doubles(c, c->a.den, nullptr, nullptr, den, order);
}

extern "C" int msmgb_copyout_gid(msmgb_ctx *c, int *gid)
{
    if (!c || !gid) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    CK(cudaMemcpyAsync(gid, c->a.gid, sizeof(int) * (size_t)c->n, cudaMemcpyDeviceToHost, c->stream), "copy-out");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    return MSMGB_OK;
}

// ---- neighbour list ---------------------------------------------------------------------------
extern "C" int msmgb_cal_neighborelist(msmgb_ctx *c)
{
    NvtxRange nvtx_range("msmgb_cal_neighborelist");
    if (!c) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    CK(cudaMemsetAsync(c->flags + kFlagMaxK, 0, sizeof(int), c->stream), "flag clear");
    RET(build_list(c));
    CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
    RET(poll_flags(c));
    c->list_valid = true;
    c->force_valid = false;
    return MSMGB_OK;
}

extern "C" int msmgb_copyout_neighborelist(msmgb_ctx *c, int *kvois, int *indi, int ld, int order)
{
    if (!c || !kvois) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    if (!c->list_valid) return set_err(c, MSMGB_ERR_ARG, "no neighbour list: call msmgb_cal_neighborelist");
    const int n = c->n, mxk = c->p.mxkvois;
    if (indi && ld < n) return set_err(c, MSMGB_ERR_ARG, "ld must be >= number of atoms");
    std::vector<int> kv((size_t)n), gid((size_t)n);
    CK(cudaMemcpy(kv.data(), c->a.kvois, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost), "copy-out");
    CK(cudaMemcpy(gid.data(), c->a.gid, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost), "copy-out");
    std::vector<int> ind;
    if (indi) {
        ind.resize((size_t)mxk * (size_t)c->a.ld);
        CK(cudaMemcpy(ind.data(), c->a.indi, sizeof(int) * ind.size(), cudaMemcpyDeviceToHost), "copy-out");
    }
    const bool sorted = order == MSMGB_ORDER_SORTED;
    for (int s = 0; s < n; ++s) {
        int g = sorted ? s : gid[(size_t)s];
        kvois[g] = kv[(size_t)s];
        if (indi)
            for (int k = 0; k < kv[(size_t)s]; ++k) {
                int j = ind[(size_t)k * (size_t)c->a.ld + (size_t)s];
                indi[(size_t)k * (size_t)ld + (size_t)g] = sorted ? j : gid[(size_t)j];
            }
    }
    return MSMGB_OK;
}

// ---- force class -----------------------------------------------------------------------------
static int ready_for_force(msmgb_ctx *c)
{
    RET(need_state(c));
    if (!c->have_tables) return set_err(c, MSMGB_ERR_ARG, "no force table: call msmgb_init_forcetable");
    RET(use_device(c));
    if (!c->list_valid) {
        CK(cudaMemsetAsync(c->flags + kFlagMaxK, 0, sizeof(int), c->stream), "flag clear");
        RET(build_list(c));
        CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
        c->list_valid = true;
    }
    return MSMGB_OK;
}

// constant external force of every active atom, from the caller-order field (XP layout)
__global__ void k_add_extfield(DevAtoms a, const double *f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || (a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) return;
    const size_t g = (size_t)a.gid[i], n = (size_t)a.n;
    a.fx[i] += f[g];
    a.fy[i] += f[n + g];
    a.fz[i] += f[2 * n + g];
}

// Cumulate_ExtForce0 (MD_ForceClass_Register_GPU.F90:584-606): the field, then every
// registered routine in order, on the forces of the force pass just enqueued
static int apply_extforces(msmgb_ctx *c)
{
    if (c->ext_field) {
        if (c->ext_field_n != c->n)
            return set_err(c, MSMGB_ERR_ARG, "the external force field was set for another atom count");
        k_add_extfield<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a, c->ext_field);
        c->launches += 1;
        RET(check_launch(c, "external force field"));
    }
    for (const auto &x : c->ext) {
        msmgb_extforce_view v;
        v.n = c->n;
        v.nbox = c->nbox;
        v.stream = (void *)c->stream;
        v.pos = (const double *)c->a.pos;
        v.fx = c->a.fx;
        v.fy = c->a.fy;
        v.fz = c->a.fz;
        v.gid = c->a.gid;
        v.ityp = c->a.ityp;
        v.statu = c->a.statu;
        v.boxid = c->a.boxid;
        const int rc = x.fn(x.user, &v);
        if (rc != 0)
            return set_err(c, MSMGB_ERR_ARG, "external force '" + x.tag + "' returned " + std::to_string(rc));
        RET(check_launch(c, "external force routine"));
    }
    return MSMGB_OK;
}

static int force_passes(msmgb_ctx *c, bool virial, bool epot)
{
    if (c->p.precision != MSMGB_PREC_FP64 && !virial && !epot) RET(need_cubic(c, "a reduced-precision force pass"));
    if (c->p.precision == MSMGB_PREC_MIXED && !virial && !epot) {
        if (c->tuned_n != c->n) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            cudaStreamIsCapturing(c->stream, &cs);
            if (cs == cudaStreamCaptureStatusNone) RET(autotune_mixed(c));
        }
        RET(launch_density32(c));
        RET(launch_force32(c));
    } else if (c->p.precision == MSMGB_PREC_FF && !virial && !epot) {
        RET(launch_density_ff(c));
        RET(launch_force_ff(c));
    } else {
        RET(launch_density(c, epot));
        RET(launch_force(c, virial));
    }
    return apply_extforces(c);
}

extern "C" int msmgb_calforce(msmgb_ctx *c)
{
    NvtxRange nvtx_range("msmgb_calforce");
    if (!c) return MSMGB_ERR_ARG;
    RET(ready_for_force(c));
    RET(force_passes(c, false, false));
    RET(poll_flags(c));
    c->force_valid = true;
    return MSMGB_OK;
}

extern "C" int msmgb_calptensor(msmgb_ctx *c, double *vt)
{
    NvtxRange nvtx_range("msmgb_calptensor");
    if (!c) return MSMGB_ERR_ARG;
    RET(ready_for_force(c));
    RET(force_passes(c, true, false));
    CK(cudaMemcpyAsync(c->h_virial, c->virial, sizeof(double) * 6 * (size_t)c->nbox, cudaMemcpyDeviceToHost,
                       c->stream), "virial copy-out");
    RET(poll_flags(c));
    c->force_valid = true;
    if (vt)
        for (int b = 0; b < c->nbox; ++b) {
            const double *v = c->h_virial + 6 * b;
            double *o = vt + 9 * b;
            o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
            o[3] = v[1]; o[4] = v[3]; o[5] = v[4];
            o[6] = v[2]; o[7] = v[4]; o[8] = v[5];
        }
    return MSMGB_OK;
}

extern "C" int msmgb_calepot(msmgb_ctx *c)
{
    NvtxRange nvtx_range("msmgb_calepot");
    if (!c) return MSMGB_ERR_ARG;
    RET(ready_for_force(c));
    RET(launch_density(c, true));
    return poll_flags(c);
}

extern "C" int msmgb_calden(msmgb_ctx *c)
{
    NvtxRange nvtx_range("msmgb_calden");
    if (!c) return MSMGB_ERR_ARG;
    RET(ready_for_force(c));
    RET(launch_density(c, false));
    return poll_flags(c);
}

extern "C" int msmgb_cal_atomic_stress(msmgb_ctx *c, double *ap, int order)
{
    NvtxRange nvtx_range("msmgb_cal_atomic_stress");
    if (!c || !ap) return MSMGB_ERR_ARG;
    RET(ready_for_force(c));
    // 72 B per atom fit in the 100 B per atom of the scratch buffer
    const size_t bytes = sizeof(double) * 9 * (size_t)c->n;
    double *tmp = (double *)c->scratch;
    RET(launch_density(c, false));
    RET(launch_stress(c, order == MSMGB_ORDER_SORTED, tmp));
    CK(cudaMemcpyAsync(ap, tmp, bytes, cudaMemcpyDeviceToHost, c->stream), "stress copy-out");
    return poll_flags(c);
}

// ---- integrator -------------------------------------------------------------------------------
extern "C" int msmgb_predictor(msmgb_ctx *c, double h)
{
    NvtxRange nvtx_range("msmgb_predictor");
    if (!c) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "the integrator"));
    RET(need_state(c));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    RET(use_device(c));
    RET(launch_vv(c, h, 0));
    c->force_valid = false;
    return poll_flags(c);
}

extern "C" int msmgb_correction(msmgb_ctx *c, double h)
{
    NvtxRange nvtx_range("msmgb_correction");
    if (!c) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "the integrator"));
    RET(need_state(c));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    RET(use_device(c));
    RET(launch_correct(c, h, false));
    return poll_flags(c);
}

// ---- step graphs with a conditional rebuild ---------------------------------------------
// A step graph is captured into a graph that owns an IF node: k_decide sets its condition on
// the device, and the node's body holds the list rebuild, so a step without a rebuild runs
// none of the rebuild kernels.
// With a two-level list the IF node runs on every rebuild and holds k_set_full, a nested IF
// node of the full rebuild (binning, sort, candidates) and the list selection from the
// candidates; a step without a rebuild evaluates that one node (two nodes in sequence cost
// 12.5 instead of ~6 us per step on a GB300).
struct RebuildNodes {
    cudaGraphConditionalHandle cond = 0, cond_inner = 0;   // single-level: cond; two-level: cond_inner
    cudaGraph_t body = nullptr, body_inner = nullptr;
};

static int begin_step_capture(msmgb_ctx *c, cudaGraph_t *g, RebuildNodes *rn)
{
    *g = nullptr;
    CK(cudaGraphCreate(g, 0), "graph create");
    cudaError_t e = two_level(c) ? cudaGraphConditionalHandleCreate(&rn->cond_inner, *g, 0, cudaGraphCondAssignDefault)
                                 : cudaGraphConditionalHandleCreate(&rn->cond, *g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(c->stream, *g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(*g);
        *g = nullptr;
        return cuda_err(c, e, "graph capture");
    }
    return MSMGB_OK;
}

// IF node at the current position of the capture; its body graph is returned for later filling
static int add_rebuild_node(msmgb_ctx *c, cudaGraphConditionalHandle cond, cudaGraph_t *body)
{
    cudaStreamCaptureStatus st;
    unsigned long long id = 0;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(c->stream, &st, &id, &cg, &deps, &edges, &nd), "capture info");
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = cond;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, cg, deps, edges, nd, &p), "conditional node");
    *body = p.conditional.phGraph_out[0];
    CK(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
       "capture dependencies");
    return MSMGB_OK;
}

// the IF node of a rebuild at the current position of the capture
static int add_rebuild_nodes(msmgb_ctx *c, RebuildNodes *rn)
{
    if (rn->cond_inner) return add_rebuild_node(c, rn->cond_inner, &rn->body_inner);
    return add_rebuild_node(c, rn->cond, &rn->body);
}

// the rebuild stage `stage` (0: the whole list build, 1: the full part of a two-level build)
// of the current atom view c->a into a conditional body; its kernel count is returned in *nk
static int fill_rebuild_body(msmgb_ctx *c, cudaGraph_t body, int stage, int64_t *nk)
{
    CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
       "graph capture");
    const int64_t l0 = c->launches;
    const int rc = stage == 0 ? build_list(c) : build_full(c);
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &out);
    *nk = c->launches - l0;
    c->launches = l0;
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(c, e, "graph capture");
    return MSMGB_OK;
}

// the body of a two-level rebuild: k_set_full, the nested IF node of the full rebuild (its
// body filled with stage 1) and the list selection (stage 2); *nk_full and *nk_inner receive
// the kernels of the nested body and of the rest
static int fill_two_level_body(msmgb_ctx *c, cudaGraph_t body, int64_t *nk_full, int64_t *nk_inner)
{
    cudaGraphConditionalHandle hf = 0;
    CK(cudaGraphConditionalHandleCreate(&hf, body, 0, cudaGraphCondAssignDefault), "conditional handle");
    CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
       "graph capture");
    const int64_t l0 = c->launches;
    cudaGraph_t full = nullptr;
    int rc = launch_set_full(c, hf);
    if (!rc) rc = add_rebuild_node(c, hf, &full);
    if (!rc) rc = build_inner(c);
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &out);
    *nk_inner = c->launches - l0;
    c->launches = l0;
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(c, e, "graph capture");
    return fill_rebuild_body(c, full, 1, nk_full);
}

// the rebuild body of one step (two-level or single-level list)
static int fill_step_rebuild(msmgb_ctx *c, const RebuildNodes &rn)
{
    c->gk_inner = 0;
    if (rn.body_inner) return fill_two_level_body(c, rn.body_inner, &c->gk_body, &c->gk_inner);
    return fill_rebuild_body(c, rn.body, 0, &c->gk_body);
}

static int finish_step_graph(msmgb_ctx *c, int rc, cudaGraph_t g, const RebuildNodes &rn, cudaGraphExec_t *out,
                             const DevAtoms &body_view)
{
    cudaGraph_t ended = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &ended);
    if (!rc && e != cudaSuccess) rc = cuda_err(c, e, "graph capture");
    if (!rc && (rn.body || rn.body_inner)) {
        const DevAtoms keep = c->a;
        c->a = body_view;
        rc = fill_step_rebuild(c, rn);
        c->a = keep;
    }
    if (!rc) {
        const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
        if (ie != cudaSuccess) {
            *out = nullptr;
            rc = cuda_err(c, ie, "graph instantiate");
        }
    }
    cudaGraphDestroy(g);
    return rc;
}

// k step bodies in one graph (msmgb_set_steps_per_graph): step s issues pre(s), the decision
// kernel with its own IF nodes (a conditional handle belongs to one node) and post(s); the
// rebuild bodies of step s work on the atom view view_after(s), the buffer step s leaves the
// state in.  *kernels receives the kernels of the k bodies outside the rebuild bodies.
template <class Pre, class Post, class View>
static int capture_k_steps(msmgb_ctx *c, int k, Pre pre, Post post, View view_after, cudaGraphExec_t *out,
                           int64_t *kernels)
{
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0), "graph create");
    std::vector<RebuildNodes> rn((size_t)k);
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < k && e == cudaSuccess; ++s)
        e = two_level(c) ? cudaGraphConditionalHandleCreate(&rn[(size_t)s].cond_inner, g, 0, cudaGraphCondAssignDefault)
                         : cudaGraphConditionalHandleCreate(&rn[(size_t)s].cond, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_err(c, e, "graph capture");
    }
    const DevAtoms base = c->a;
    const int64_t l0 = c->launches;
    int rc = MSMGB_OK;
    for (int s = 0; s < k && !rc; ++s) {
        rc = pre(s);
        if (!rc) rc = launch_decide(c, c->p.skin_trigger, c->p.nb_uptab, rn[(size_t)s].cond, true,
                                    rn[(size_t)s].cond_inner);
        if (!rc) rc = add_rebuild_nodes(c, &rn[(size_t)s]);
        if (!rc) rc = post(s);
        c->a = base;
    }
    *kernels = c->launches - l0;
    c->launches = l0;
    cudaGraph_t ended = nullptr;
    e = cudaStreamEndCapture(c->stream, &ended);
    if (!rc && e != cudaSuccess) rc = cuda_err(c, e, "graph capture");
    for (int s = 0; s < k && !rc; ++s) {
        c->a = view_after(s);
        rc = fill_step_rebuild(c, rn[(size_t)s]);
        c->a = base;
    }
    if (!rc) {
        e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) {
            *out = nullptr;
            rc = cuda_err(c, e, "graph instantiate");
        }
    }
    cudaGraphDestroy(g);
    return rc;
}

static int capture_step(msmgb_ctx *c, double h)
{
    free_graph(c);
    cudaGraph_t g = nullptr;
    RebuildNodes rn;
    RET(begin_step_capture(c, &g, &rn));
    int64_t l0 = c->launches;
    int rc = launch_vv(c, h, 1);
    if (!rc) rc = launch_decide(c, c->p.skin_trigger, c->p.nb_uptab, rn.cond, true, rn.cond_inner);
    if (!rc) rc = add_rebuild_nodes(c, &rn);
    if (!rc) rc = force_passes(c, false, false);
    const int64_t nk = c->launches - l0;
    RET(finish_step_graph(c, rc, g, rn, &c->step_graph, c->a));
    c->graph_kernels = nk;
    c->launches = l0;
    if (c->steps_per_graph > 1) {
        const DevAtoms base = c->a;
        RET(capture_k_steps(
            c, c->steps_per_graph, [&](int) { return launch_vv(c, h, 1); },
            [&](int) { return force_passes(c, false, false); }, [&](int) { return base; }, &c->step_graphk,
            &c->graph_kernels_k));
    }
    c->graph_h = h;
    c->graph_prec = c->p.precision;
    c->graph_n = c->n;
    c->graph_tune = c->tune_dens_unroll * 64 + c->tune_force_unroll;
    return MSMGB_OK;
}

// ---- fused step: force pass + integrator in one kernel (mixed single species, float-float)
static bool fused_mixed(const msmgb_ctx *c)
{
    // external forces go between the force pass and the corrector: the unfused step then
    return (c->p.precision == MSMGB_PREC_MIXED || c->p.precision == MSMGB_PREC_FF) && c->ext.empty() &&
           !c->ext_field;
}

static int step_density(msmgb_ctx *c)
{
    return c->p.precision == MSMGB_PREC_FF ? launch_density_ff(c) : launch_density32(c);
}

static int step_force_vv(msmgb_ctx *c, double h)
{
    return c->p.precision == MSMGB_PREC_FF ? launch_force_ff_vv(c, h) : launch_force32_vv(c, h);
}

static int step_force(msmgb_ctx *c)
{
    return c->p.precision == MSMGB_PREC_FF ? launch_force_ff(c) : launch_force32(c);
}

// atom view whose positions are buffer p (0: c->a's own, 1: the second buffer) and whose
// next-step positions are the other buffer
static DevAtoms atoms_on(const msmgb_ctx *c, const DevAtoms &base, int p)
{
    DevAtoms a = base;
    a.pos = p ? c->pos2 : base.pos;
    a.posff = p ? c->posff2 : base.posff;
    a.pos_nxt = p ? base.pos : c->pos2;
    a.posff_nxt = p ? base.posff : c->posff2;
    return a;
}

static int end_capture(msmgb_ctx *c, int rc, cudaGraphExec_t *out)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_err(c, e, "graph capture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { *out = nullptr; return cuda_err(c, e, "graph instantiate"); }
    return MSMGB_OK;
}

// Graphs of the fused mixed step: PRE (predictor of step 1, decision, rebuild), LOOP[p]
// (density on buffer p, force + corrector n + predictor n+1 into buffer 1-p, decision,
// rebuild of buffer 1-p) and FINAL[p] (density, force, corrector of the last step).
static int capture_fused(msmgb_ctx *c, double h)
{
    free_graph(c);
    if (!c->pos2) {
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        CK(dalloc(&c->pos2, (size_t)c->cap_atoms), "cudaMalloc second position buffer");
        CK(dalloc(&c->posff2, (size_t)c->cap_atoms), "cudaMalloc second position buffer");
    }
    const DevAtoms base = c->a;
    int rc = MSMGB_OK;
    // tune the fused mixed kernel on the current state (h = 0 changes nothing), outside
    // capture, once per atom count (a new state of the same size keeps the choice)
    if (c->p.precision == MSMGB_PREC_MIXED && c->tuned_fused_n != c->n) {
        c->a = atoms_on(c, base, 0);
        rc = autotune_fused(c);
        c->a = base;
        RET(rc);
    }
    const int64_t l_start = c->launches;
    int64_t l0 = c->launches;
    {
        cudaGraph_t g = nullptr;
        RebuildNodes rn;
        RET(begin_step_capture(c, &g, &rn));
        c->a = atoms_on(c, base, 0);
        rc = launch_vv(c, h, 0);
        if (!rc) rc = launch_decide(c, c->p.skin_trigger, c->p.nb_uptab, rn.cond, true, rn.cond_inner);
        if (!rc) rc = add_rebuild_nodes(c, &rn);
        c->gk_pre = c->launches - l0;
        rc = finish_step_graph(c, rc, g, rn, &c->g_pre, atoms_on(c, base, 0));
        c->a = base;
        RET(rc);
    }
    for (int p = 0; p < 2; ++p) {
        l0 = c->launches;
        cudaGraph_t g = nullptr;
        RebuildNodes rn;
        RET(begin_step_capture(c, &g, &rn));
        c->a = atoms_on(c, base, p);
        rc = step_density(c);
        if (!rc) rc = step_force_vv(c, h);
        if (!rc) rc = launch_decide(c, c->p.skin_trigger, c->p.nb_uptab, rn.cond, true, rn.cond_inner);
        if (!rc) rc = add_rebuild_nodes(c, &rn);
        c->gk_loop = c->launches - l0;
        rc = finish_step_graph(c, rc, g, rn, &c->g_loop[p], atoms_on(c, base, 1 - p));
        c->a = base;
        RET(rc);
        l0 = c->launches;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        c->a = atoms_on(c, base, p);
        rc = step_density(c);
        if (!rc) rc = step_force(c);
        if (!rc) rc = launch_correct(c, h, false);
        c->a = base;
        RET(end_capture(c, rc, &c->g_final[p]));
        c->gk_final = c->launches - l0;
    }
    if (c->steps_per_graph > 1) {
        for (int p = 0; p < 2; ++p) {
            rc = capture_k_steps(
                c, c->steps_per_graph,
                [&](int st) {
                    c->a = atoms_on(c, base, (p + st) & 1);
                    int r = step_density(c);
                    return r ? r : step_force_vv(c, h);
                },
                [&](int) { return MSMGB_OK; }, [&](int st) { return atoms_on(c, base, 1 - ((p + st) & 1)); },
                &c->g_loopk[p], &c->gk_loopk);
            c->a = base;
            RET(rc);
        }
    }
    c->launches = l_start;            // capturing launches nothing; graph launches are counted
    c->fg_h = h;
    c->fg_n = c->n;
    c->fg_prec = c->p.precision;
    c->fg_tune = c->tune_dens_unroll * 64 + c->tune_force_unroll;
    return MSMGB_OK;
}

static int ensure_graphs(msmgb_ctx *c, double h)
{
    if (c->graphs_stale) {
        free_graph(c);
        c->graphs_stale = false;
    }
    if (fused_mixed(c)) {
        if (!c->g_pre || c->fg_h != h || c->fg_n != c->n || c->fg_prec != c->p.precision ||
            c->fg_tune != c->tune_dens_unroll * 64 + c->tune_force_unroll)
            return capture_fused(c, h);
        return MSMGB_OK;
    }
    if (!c->step_graph || c->graph_h != h || c->graph_prec != c->p.precision || c->graph_n != c->n ||
        c->graph_tune != c->tune_dens_unroll * 64 + c->tune_force_unroll)
        return capture_step(c, h);
    return MSMGB_OK;
}

// kernels run by the conditional rebuild bodies since the rebuild counters were cleared
// (h_flags freshly read): every rebuild runs the first body, or with a two-level list the
// selection body, and the full rebuilds also the first one
static void count_rebuild_kernels(msmgb_ctx *c)
{
    const int64_t nreb = c->h_flags[kFlagRebuilds];
    const int64_t nfull = c->gk_inner > 0 ? (int64_t)c->h_flags[kFlagFull] : nreb;
    if (c->gk_inner > 0) c->launches += nreb * c->gk_inner + nfull * c->gk_body;
    else c->launches += nreb * c->gk_body;
    c->step_rebuilds += nreb;
    c->step_full += nfull;
}

extern "C" int msmgb_rebuild_counts(const msmgb_ctx *c, int64_t *rebuilds, int64_t *full)
{
    if (!c) return MSMGB_ERR_ARG;
    if (rebuilds) *rebuilds = c->step_rebuilds;
    if (full) *full = c->step_full;
    return MSMGB_OK;
}

// issues nsteps complete steps (the fused path ends with its own corrector)
static int issue_steps(msmgb_ctx *c, int nsteps, double h)
{
    if (nsteps <= 0) return MSMGB_OK;
    const int k = c->steps_per_graph;
    if (!fused_mixed(c)) {
        for (int s = 0; s < nsteps;) {
            if (k > 1 && c->step_graphk && nsteps - s >= k) {
                CK(cudaGraphLaunch(c->step_graphk, c->stream), "graph launch");
                c->launches += c->graph_kernels_k;
                s += k;
            } else {
                CK(cudaGraphLaunch(c->step_graph, c->stream), "graph launch");
                c->launches += c->graph_kernels;
                ++s;
            }
            ++c->graph_launches;
        }
        return MSMGB_OK;
    }
    CK(cudaGraphLaunch(c->g_pre, c->stream), "graph launch");
    c->launches += c->gk_pre;
    ++c->graph_launches;
    int p = 0;
    for (int s = 1; s < nsteps;) {
        if (k > 1 && c->g_loopk[p] && nsteps - s >= k) {
            CK(cudaGraphLaunch(c->g_loopk[p], c->stream), "graph launch");
            c->launches += c->gk_loopk;
            s += k;
            p = (p + k) & 1;
        } else {
            CK(cudaGraphLaunch(c->g_loop[p], c->stream), "graph launch");
            c->launches += c->gk_loop;
            p ^= 1;
            ++s;
        }
        ++c->graph_launches;
    }
    CK(cudaGraphLaunch(c->g_final[p], c->stream), "graph launch");
    c->launches += c->gk_final;
    ++c->graph_launches;
    if (p) {   // the state ended in the second buffer: bring it back to the primary one
        CK(cudaMemcpyAsync(c->a.pos, c->pos2, sizeof(double4_32a) * (size_t)c->n, cudaMemcpyDeviceToDevice,
                           c->stream), "position copy");
        CK(cudaMemcpyAsync(c->a.posff, c->posff2, sizeof(PosFF) * (size_t)c->n, cudaMemcpyDeviceToDevice,
                           c->stream), "position copy");
    }
    return MSMGB_OK;
}

extern "C" int msmgb_run_steps(msmgb_ctx *c, int nsteps, double h, int *rebuilds)
{
    NvtxRange nvtx_range("msmgb_run_steps");
    if (!c || nsteps < 0) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "MD"));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    RET(ready_for_force(c));
    if (!c->force_valid) {
        RET(force_passes(c, false, false));
        c->force_valid = true;
    }
    CK(cudaMemsetAsync(c->flags + kFlagRebuilds, 0, sizeof(int) * 3, c->stream), "flag clear");  // rebuilds, pending, step
    CK(cudaMemsetAsync(c->flags + kFlagFull, 0, sizeof(int), c->stream), "flag clear");
    RET(ensure_graphs(c, h));
    RET(issue_steps(c, nsteps, h));
    RET(launch_correct(c, h, true));          // no-op unless the last step left a pending half-kick
    int rc = poll_flags(c);
    if (rebuilds) *rebuilds = c->h_flags[kFlagRebuilds];
    count_rebuild_kernels(c);
    CK(cudaMemsetAsync(c->flags + kFlagRebuilds, 0, sizeof(int), c->stream), "flag clear");
    CK(cudaMemsetAsync(c->flags + kFlagFull, 0, sizeof(int), c->stream), "flag clear");
    return rc;
}

// asynchronous variant for timing loops: no host synchronisation; nsteps = 0 only prepares
// the list, the forces and the step graphs
extern "C" int msmgb_enqueue_steps(msmgb_ctx *c, int nsteps, double h)
{
    NvtxRange nvtx_range("msmgb_enqueue_steps");
    if (!c || nsteps < 0) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "MD"));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    RET(ready_for_force(c));
    if (!c->force_valid) {
        RET(force_passes(c, false, false));
        c->force_valid = true;
    }
    RET(ensure_graphs(c, h));
    return issue_steps(c, nsteps, h);
}

extern "C" int msmgb_finish_steps(msmgb_ctx *c, double h, int *rebuilds)
{
    NvtxRange nvtx_range("msmgb_finish_steps");
    if (!c) return MSMGB_ERR_ARG;
    RET(use_device(c));
    RET(launch_correct(c, h, true));
    int rc = poll_flags(c);
    if (rebuilds) *rebuilds = c->h_flags[kFlagRebuilds];
    count_rebuild_kernels(c);
    CK(cudaMemsetAsync(c->flags + kFlagRebuilds, 0, sizeof(int), c->stream), "flag clear");
    CK(cudaMemsetAsync(c->flags + kFlagFull, 0, sizeof(int), c->stream), "flag clear");
    return rc;
}

// ---- differentiation ------------------------------------------------------------------------
static int ensure_hvp_pair(msmgb_ctx *c)
{
    if (c->hvp_pair) return MSMGB_OK;
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    CK(cudaMalloc(&c->hvp_pair, sizeof(double) * 5 * (size_t)c->a.ld * (size_t)c->p.mxkvois),
       "HVP pair buffer");
    return MSMGB_OK;
}

extern "C" int msmgb_hvp(msmgb_ctx *c, const double *v, double *hv)
{
    NvtxRange nvtx_range("msmgb_hvp");
    if (!c || !v || !hv) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "the Hessian-vector product"));
    RET(ready_for_force(c));
    RET(ensure_hvp_pair(c));
    const int n = c->n;
    const size_t N = (size_t)c->cap_atoms;
    char *s = (char *)c->scratch;
    double *v4 = (double *)s;                 // 32 B per atom
    double *dd = (double *)(s + 32 * N);      // 16 B: F'(rho) and its directional derivative
    double *hvs = (double *)(s + 48 * N);     // 24 B, sorted SoA result
    double *io = (double *)(s + 72 * N);      // 24 B, caller-order staging (input, then output)
    CK(cudaMemcpyAsync(io, v, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, c->stream), "hvp copy-in");
    RET(launch_hvp(c, io, hvs, v4, dd));
    k_unpack3<<<nblk(n, kBlock), kBlock, 0, c->stream>>>(hvs, hvs + n, hvs + 2 * (size_t)n, c->a.gid, n, 0, io);
    c->launches += 1;
    RET(check_launch(c, "hvp copy-out"));
    CK(cudaMemcpyAsync(hv, io, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, c->stream), "hvp copy-out");
    return poll_flags(c);
}

extern "C" int msmgb_cr_param_tables(const double *prm, double rmax, int ntab, double *d);

extern "C" int msmgb_param_adjoint(msmgb_ctx *c, int pot, const double *prm, const double *ft,
                                   double *loss, double *grad)
{
    NvtxRange nvtx_range("msmgb_param_adjoint");
    if (!c || !prm || !ft || !grad) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "the parameter adjoint"));
    if (pot != MSMGB_POT_CR) return set_err(c, MSMGB_ERR_ARG, "the adjoint supports the Cleri-Rosato parameters");
    RET(ready_for_force(c));
    if (c->tab.pottype != MSMGB_FS_TYPE || c->tab.nkind != 1 || c->tab.ngroup != 1)
        return set_err(c, MSMGB_ERR_ARG, "the adjoint needs single-species FS tables");
    const int n = c->n, ntab = c->tab.ntab;
    const size_t ntp = (size_t)c->tab.ntp, N = (size_t)c->cap_atoms;
    // parameter-derivative tables, padded like the force tables
    std::vector<double> raw((size_t)15 * ntab), pad((size_t)15 * ntp, 0.0);
    RET(msmgb_cr_param_tables(prm, c->tab_rmax, ntab, raw.data()));
    for (int r = 0; r < 15; ++r) {
        double *row = pad.data() + (size_t)r * ntp;
        for (int i = 1; i <= ntab; ++i) row[i] = raw[(size_t)r * ntab + (i - 1)];
        row[ntab + 1] = row[ntab];
    }
    const size_t need = pad.size() * sizeof(double) + 8 * sizeof(double);
    if (c->adj_bytes < need) {
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        if (c->adj_mem) cudaFree(c->adj_mem);
        c->adj_mem = nullptr;
        CK(cudaMalloc(&c->adj_mem, need), "adjoint alloc");
        c->adj_bytes = need;
    }
    double *dtab = (double *)c->adj_mem;
    double *acc = dtab + pad.size();
    CK(cudaMemcpyAsync(dtab, pad.data(), pad.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream),
       "adjoint upload");
    char *s = (char *)c->scratch;
    double *w4 = (double *)s;                  // 32 B per atom
    double *dd = (double *)(s + 32 * N);       // 5 x 8 B
    double *io = (double *)(s + 72 * N);       // 24 B: target forces, caller order
    CK(cudaMemcpyAsync(io, ft, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, c->stream), "adjoint copy-in");
    RET(launch_density(c, false));             // FP64 forces at the current parameters
    RET(launch_force(c, false));
    RET(launch_adjoint(c, io, dtab, w4, dd, acc));
    double h[6];
    CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "adjoint copy-out");
    RET(poll_flags(c));
    c->force_valid = true;
    c->den_is32 = false;
    for (int m = 0; m < 5; ++m) grad[m] = 2.0 * h[m];
    if (loss) *loss = h[5];
    return MSMGB_OK;
}

// ---- timing helpers (CUDA events on the context stream) -------------------------------------
extern "C" int msmgb_time_steps(msmgb_ctx *c, int nsteps, double h, float *ms, int *rebuilds)
{
    if (!c || !ms || nsteps < 1) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "MD"));
    RET(msmgb_enqueue_steps(c, 0, h));           // list, forces and the step graph are ready
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    CK(cudaEventRecord(e0, c->stream), "event");
    int rc = msmgb_enqueue_steps(c, nsteps, h);
    CK(cudaEventRecord(e1, c->stream), "event");
    CK(cudaEventSynchronize(e1), "event");
    CK(cudaEventElapsedTime(ms, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    return msmgb_finish_steps(c, h, rebuilds);
}

// Average device time (ms) of one launch of each pass: out[0] density, out[1] force,
// out[2] full list rebuild, out[3] integrator (timed with h = 0 so the state is unchanged
// while the memory traffic is that of a real step), out[4] the fused mixed force pass +
// integrator of the step graph (h = 0 as well; 0 when the fused step is not in use).
extern "C" int msmgb_time_passes(msmgb_ctx *c, int reps, float *out)
{
    if (!c || !out || reps < 1) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "pass timing"));      // it times the integrator and the step kernels
    RET(ready_for_force(c));
    if (!c->have_masses) return set_err(c, MSMGB_ERR_ARG, "no masses: call msmgb_set_masses");
    const bool mixed = c->p.precision == MSMGB_PREC_MIXED;
    const bool ffp = c->p.precision == MSMGB_PREC_FF;
    const bool fused = fused_mixed(c) && c->pos2;
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]), "event");
    CK(cudaEventCreate(&ev[1]), "event");
    out[4] = 0.0f;
    for (int which = 0; which < 5; ++which) {
        if (which == 4 && !fused) break;
        // the fused kernel reads the {position, F'(rho)} records of the density pass:
        // refresh them for the current positions (untimed)
        if (which == 4) RET(step_density(c));
        double total = 0.0;
        for (int r = 0; r < reps + 1; ++r) {
            CK(cudaStreamSynchronize(c->stream), "synchronize");
            CK(cudaEventRecord(ev[0], c->stream), "event");
            int rc = MSMGB_OK;
            if (which == 0) rc = mixed ? launch_density32(c) : (ffp ? launch_density_ff(c) : launch_density(c, false));
            else if (which == 1) rc = mixed ? launch_force32(c) : (ffp ? launch_force_ff(c) : launch_force(c, false));
            else if (which == 2) rc = build_list(c);
            else if (which == 3) rc = launch_vv(c, 0.0, 2);
            else {
                const DevAtoms base = c->a;
                c->a = atoms_on(c, base, 0);
                rc = step_force_vv(c, 0.0);
                c->a = base;
            }
            if (rc) return rc;
            CK(cudaEventRecord(ev[1], c->stream), "event");
            CK(cudaEventSynchronize(ev[1]), "event");
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[0], ev[1]), "event");
            if (r > 0) total += ms;                    // first launch is a warm-up
            if (which == 2) {
                // the rebuild re-sorted the atoms: the forces must follow
                RET(force_passes(c, false, false));
            }
        }
        out[which] = (float)(total / reps);
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    CK(cudaMemsetAsync(c->maxdisp, 0, sizeof(unsigned long long), c->stream), "flag clear");
    return poll_flags(c);
}

// largest neighbour count of the last list build and the mean count, for the byte model
extern "C" int msmgb_list_stats(msmgb_ctx *c, int *maxk, double *meank)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    std::vector<int> kv((size_t)c->n);
    CK(cudaMemcpy(kv.data(), c->a.kvois, sizeof(int) * (size_t)c->n, cudaMemcpyDeviceToHost), "copy-out");
    long s = 0;
    int m = 0;
    for (int k : kv) { s += k; m = std::max(m, k); }
    if (maxk) *maxk = m;
    if (meank) *meank = (double)s / (double)c->n;
    return MSMGB_OK;
}

// float-float record of each active atom against its FP64 position (msmgb_check_records):
// the error in units of the quantum as the bits of a non-negative double (ordered like the
// values), and the atoms whose hi is off the quantum or whose |lo| exceeds half of it
__global__ void k_check_records(DevAtoms a, unsigned long long *worst, int *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || (a.statu[i] & MSMGB_STATU_ACTIVE) != MSMGB_STATU_ACTIVE) return;
    const DevBox &b = a.box[a.boxid[i]];
    const PosFF f = ld_ff(a.posff + i);
    const double4_32a p = a.pos[i];
    const double x[3] = {p.x, p.y, p.z};
    const float h[3] = {f.hx, f.hy, f.hz}, l[3] = {f.lx, f.ly, f.lz};
    const double q = (double)b.qq;
    double e = 0.0;
    int broken = 0;
    for (int k = 0; k < 3; ++k) {
        const double m = (double)h[k] / q;
        if (m != rint(m) || fabs((double)l[k]) > 0.5 * q) broken = 1;
        e = fmax(e, fabs(((double)h[k] - (x[k] + b.ushift[k])) + (double)l[k]) / q);
    }
    if (broken) atomicAdd(bad, 1);
    if (e > 0.0) atomicMax(worst, (unsigned long long)__double_as_longlong(e));
}

extern "C" int msmgb_check_records(msmgb_ctx *c, double *max_err, int *violations)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    unsigned long long *w = nullptr;
    CK(cudaMalloc((void **)&w, 2 * sizeof(unsigned long long)), "cudaMalloc check");
    cudaError_t e = cudaMemsetAsync(w, 0, 2 * sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) {
        k_check_records<<<(c->n + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(c->a, w, (int *)(w + 1));
        e = cudaGetLastError();
    }
    unsigned long long hw[2] = {0ull, 0ull};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hw, w, sizeof(hw), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(w);
    if (e != cudaSuccess) return cuda_err(c, e, "record check");
    c->launches += 1;
    if (max_err) std::memcpy(max_err, &hw[0], sizeof(double));   // bits of a non-negative double
    if (violations) *violations = (int)(unsigned)hw[1];
    return MSMGB_OK;
}

extern "C" int msmgb_tile_stats(msmgb_ctx *c, int *blocks, int *tiled, double *mean_halo, int *max_halo)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(need_state(c));
    RET(use_device(c));
    const int nb = (c->n + kBlock - 1) / kBlock;
    int t = 0, mx = 0;
    double s = 0.0;
    if (c->halo_on && c->list_valid && c->a.hmeta) {
        std::vector<int2> m((size_t)nb);
        CK(cudaStreamSynchronize(c->stream), "synchronize");
        CK(cudaMemcpy(m.data(), c->a.hmeta, sizeof(int2) * (size_t)nb, cudaMemcpyDeviceToHost), "copy-out");
        for (const int2 &q : m)
            if (q.x >= 0) { ++t; s += q.y; mx = std::max(mx, q.y); }
    }
    if (blocks) *blocks = nb;
    if (tiled) *tiled = t;
    if (mean_halo) *mean_halo = t ? s / t : 0.0;
    if (max_halo) *max_halo = mx;
    return MSMGB_OK;
}

// Device time of one Hessian-vector product (gather of v + the two HVP passes) and of one
// FP64 force call (density + force pass) on the current state, averaged over `reps`
// launches after a warm-up; v (caller order, XP layout) is uploaded once before timing.
extern "C" int msmgb_time_hvp(msmgb_ctx *c, const double *v, int reps, float *ms_hvp, float *ms_force)
{
    if (!c || !v || !ms_hvp || !ms_force || reps < 1) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "the Hessian-vector product"));
    RET(ready_for_force(c));
    RET(ensure_hvp_pair(c));
    const int n = c->n;
    const size_t N = (size_t)c->cap_atoms;
    char *s = (char *)c->scratch;
    double *v4 = (double *)s, *dd = (double *)(s + 32 * N), *hvs = (double *)(s + 48 * N);
    double *io = (double *)(s + 72 * N);
    CK(cudaMemcpyAsync(io, v, sizeof(double) * 3 * (size_t)n, cudaMemcpyDefault, c->stream), "hvp copy-in");
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    float t[2] = {0.f, 0.f};
    for (int which = 0; which < 2; ++which) {
        for (int r = 0; r < reps + 1; ++r) {
            if (r == 1) CK(cudaEventRecord(e0, c->stream), "event");
            if (which == 0) RET(launch_hvp(c, io, hvs, v4, dd));
            else { RET(launch_density(c, false)); RET(launch_force(c, false)); }
        }
        CK(cudaEventRecord(e1, c->stream), "event");
        CK(cudaEventSynchronize(e1), "event");
        CK(cudaEventElapsedTime(&t[which], e0, e1), "event");
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_hvp = t[0] / reps;
    *ms_force = t[1] / reps;
    c->force_valid = true;
    return poll_flags(c);
}

// Launch variants chosen by the autotuner: out[0] density unroll, out[1] force unroll;
// ms[0], ms[1]: their measured time per launch (0 before tuning).
extern "C" int msmgb_selftest_wait(msmgb_ctx *c)
{
    if (!c) return MSMGB_ERR_ARG;
    RET(use_device(c));
    RET(launch_wait_selftest(c));
    return poll_flags(c);
}

extern "C" int msmgb_set_tuning(msmgb_ctx *c, const int *codes)
{
    if (!c || !codes) return MSMGB_ERR_ARG;
    static const int valid_d[] = {1, 2, 3, 4, 5, 9, 10, 18, 19, 20, 21, 66, 68, 82, 84};
    static const int valid_f[] = {1, 2, 3, 4, 5, 9, 10, 18, 19, 20, 21, 50, 51, 52, 53};
    auto in = [](int v, const int *set, int n) {
        for (int k = 0; k < n; ++k)
            if (set[k] == v) return true;
        return false;
    };
    const bool multi = c->tab.ngroup > 1;
    // density +128 (128-thread blocks) on the one-thread-per-atom families only
    const int d = codes[0];
    // +256 (single kind): the table-assisted density pass, 2-5 in the low bits, +16, +128
    // +512: one box, its constants as a kernel parameter
    const bool d_q = !multi && d >= 0 && (d & 256) && (d & ~(512 | 256 | 128 | 16 | 7)) == 0 && (d & 7) >= 2 &&
                     (d & 7) <= 5 && (!(d & 512) || c->nbox == 1);
    const bool d_ok = d < 0 || d_q || in(d, valid_d, 15) ||
                      ((d & 128) && (d & ~128) < 32 && (d & 8) == 0 && in(d & ~128, valid_d, 15));
    // fused: 0-23 (several kinds 0-3), + 32 for 0-17 (0-3) in 128-thread blocks
    const int u = codes[2];
    const bool u_sb = !multi && c->nbox == 1 && u >= 64 && u < 128 && ((u & ~32) - 64) >= 12 &&
                      ((u & ~32) - 64) < 18;
    // +128 (single kind, fixed-point records on): 12-17, +32, +64 (one box)
    const int ub = u & ~(128 | 64 | 32);
    const bool u_fix = !multi && c->a.fix_on && u >= 128 && u < 256 && ub >= 12 && ub < 18 &&
                       (!(u & 64) || c->nbox == 1);
    const bool u_ok = u < 0 || u_sb || u_fix || u < (multi ? 4 : 24) || (u >= 32 && u < 32 + (multi ? 4 : 18));
    // force +128 (single kind, fixed-point records on): the batched codes 50-53
    const int f = codes[1];
    const bool f_fix = !multi && c->a.fix_on && f >= 128 && f < 256 && (f - 128) >= 50 && (f - 128) <= 53;
    if (!d_ok || (f >= 0 && !f_fix && !in(f, valid_f, 15)) || !u_ok)
        return set_err(c, MSMGB_ERR_ARG, "unknown kernel variant code");
    if (((codes[0] >= 0 && (codes[0] & 64)) || (codes[2] >= 20 && codes[2] < 24)) &&
        (c->tab.ngroup > 1 || c->p.precision != MSMGB_PREC_MIXED))
        return set_err(c, MSMGB_ERR_ARG, "cell-tile variants need one table kind and MIXED precision");
    if ((codes[2] == 18 || codes[2] == 19) && c->tab.ngroup == 1) {
        RET(use_device(c));
        if (ensure_list_maps(c) != 1) return set_err(c, MSMGB_ERR_ARG, "TMA list descriptors unavailable");
    }
    if (codes[0] >= 0 || codes[1] >= 0) {
        if (codes[0] >= 0) c->tune_dens_unroll = codes[0];
        if (codes[1] >= 0) c->tune_force_unroll = codes[1];
        c->tuned_n = c->n;
    }
    if (codes[2] >= 0) {
        c->tune_fused = codes[2];
        c->tuned_fused_n = c->n;
    }
    free_graph(c);
    if (uses_tiles(c)) {
        RET(use_device(c));
        RET(enable_halo(c));
    } else {
        c->halo_on = false;
    }
    return MSMGB_OK;
}

extern "C" int msmgb_set_outer_skin(msmgb_ctx *c, double skin)
{
    if (!c) return MSMGB_ERR_ARG;
    if (!(skin >= 0.0 && skin <= c->p.rc_nl))
        return set_err(c, MSMGB_ERR_ARG, "the outer skin must lie in [0, rc_nl]");
    if (skin != c->outer_skin) {
        c->outer_skin = skin;
        free_graph(c);
        c->list_valid = false;        // the next list build is a full one (candidates included)
    }
    return MSMGB_OK;
}

extern "C" int msmgb_set_boxshape(msmgb_ctx *c, int ibox, const double *bs)
{
    if (!c || !bs || ibox < 0 || ibox >= c->cap_boxes) return MSMGB_ERR_ARG;
    for (int q = 0; q < 9; ++q)
        if (!std::isfinite(bs[q])) return set_err(c, MSMGB_ERR_ARG, "BOXSHAPE must be finite");
    if (c->shapes.size() < (size_t)c->cap_boxes * 9) {
        const size_t old = c->shapes.size() / 9;
        c->shapes.resize((size_t)c->cap_boxes * 9, 0.0);
        for (size_t b = old; b < (size_t)c->cap_boxes; ++b)
            c->shapes[b * 9] = c->shapes[b * 9 + 4] = c->shapes[b * 9 + 8] = 1.0;
    }
    memcpy(&c->shapes[(size_t)ibox * 9], bs, sizeof(double) * 9);
    return MSMGB_OK;
}

// Device time of a full list rebuild and of a list selection from the candidates (two-level
// list; 0 without one), averaged over `reps` launches after a warm-up.
extern "C" int msmgb_time_rebuilds(msmgb_ctx *c, int reps, float *full_ms, float *inner_ms)
{
    if (!c || !full_ms || !inner_ms || reps < 1) return MSMGB_ERR_ARG;
    RET(need_cubic(c, "rebuild timing"));   // rebuilds inside MD steps need cubic boxes
    RET(ready_for_force(c));
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]), "event");
    CK(cudaEventCreate(&ev[1]), "event");
    float out[2] = {0.0f, 0.0f};
    for (int which = 0; which < 2; ++which) {
        if (which == 1 && !two_level(c)) break;
        double total = 0.0;
        for (int r = 0; r < reps + 1; ++r) {
            CK(cudaEventRecord(ev[0], c->stream), "event");
            RET(which == 0 ? build_list(c) : build_inner(c));
            CK(cudaEventRecord(ev[1], c->stream), "event");
            CK(cudaEventSynchronize(ev[1]), "event");
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[0], ev[1]), "event");
            if (r > 0) total += ms;
        }
        out[which] = (float)(total / reps);
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    c->force_valid = false;            // a full rebuild re-sorts the atoms
    *full_ms = out[0];
    *inner_ms = out[1];
    return poll_flags(c);
}

extern "C" int msmgb_get_tuning(const msmgb_ctx *c, int *out, float *ms)
{
    if (!c || !out) return MSMGB_ERR_ARG;
    out[0] = c->tune_dens_unroll;
    out[1] = c->tune_force_unroll;
    out[2] = c->tune_fused;
    if (ms) { ms[0] = c->tune_ms[0]; ms[1] = c->tune_ms[1]; ms[2] = c->tune_ms_fused; }
    return MSMGB_OK;
}
