// noalloc.cu -- a force call that allocates no device memory.
//
// Every other entry point of this library works through a context, and creating a context
// allocates device memory with cudaMalloc.  Some callers cannot do that: a host code whose
// device memory is already laid out and owned by its own runtime (msmpscu's CUDA Fortran
// host keeps positions, lists and forces in its own device arrays), a code that runs under
// a fixed device-memory budget handed out by its own allocator, or one that must not let
// cudaMalloc's implicit device synchronisation stall its other streams in the middle of a
// time step.  msmgb_calforce_noalloc serves them: the caller passes device pointers to its
// inputs and its output, and the only other memory the call needs -- F'(rho) of every atom
// between the density pass and the force pass, plus one error word -- lives in arrays
// declared at file scope below.  They are part of the library image: every GPU on which the
// library is used holds them (8 MiB + 256 B) until the process exits.
//
// The host cannot use the names of those arrays as device addresses (in host code the name
// is a host-side stand-in), so the first call on each device, with that device current,
// looks the addresses up with cudaGetSymbolAddress and keeps them for later calls.  Under
// CUDA's lazy module loading (the default) that lookup is also what loads this library's
// device code onto the device, with the synchronisation a module load implies; a caller
// that must avoid it mid-step makes one call at set-up (a call with n = 1 will do).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "msmgb_internal.cuh"

namespace {

constexpr int kNoAllocMaxAtoms = MSMGB_NOALLOC_MAX_ATOMS;
constexpr int kMaxDevices = 64;

// F'(rho) per atom, shared by every call on this device (contents persist between calls)
static __device__ __align__(256) double g_den_scratch[kNoAllocMaxAtoms];
// error bits of the running call (bit 0: density beyond the F(rho) table; bit 1: a
// neighbour id outside 0..n-1, whose slot is skipped); cleared at the start of every call
static __device__ __align__(256) int g_err_scratch[64];

struct DevScratch {
    bool ready = false;
    double *den = nullptr;
    int *err = nullptr;
};
DevScratch g_dev[kMaxDevices];
std::mutex g_setup_mutex;

void put_msg(const msmgb_force_noalloc *a, const char *msg)
{
    if (a && a->errbuf && a->errlen > 0) {
        strncpy(a->errbuf, msg, (size_t)a->errlen - 1);
        a->errbuf[a->errlen - 1] = '\0';
    }
}

__device__ __forceinline__ double mi(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

// table in the reference's layout, 1-based point i at T[i-1]; KK = NTAB reads NTAB again
// for the upper point (only ever weighted by DK = 0), KK = 0 reads 0
__device__ __forceinline__ double lerp_ref(const double *__restrict__ T, int ntab, int kk, double dk)
{
    double a = kk >= 1 ? __ldg(T + min(kk, ntab) - 1) : 0.0;
    double b = kk + 1 >= 1 ? __ldg(T + min(kk + 1, ntab) - 1) : 0.0;
    return a + dk * (b - a);
}

struct NaArgs {
    int n, ld, ntab, nembd, pottype;
    const double *x, *y, *z;
    const int *statu, *kvois, *indi;
    double len[3], half[3];
    int ifpd[3];
    double csi, ru2, rhod;
    const double *potb, *fpotr, *fpotb, *dfembd;
    double *fp;
};

__global__ void __launch_bounds__(256) k_na_density(NaArgs a, double *den, int *err)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double rho = 0.0;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const double px = a.x[i], py = a.y[i], pz = a.z[i];
        const int kn = a.kvois[i];
        for (int w = 0; w < kn; ++w) {
            int j = __ldg(a.indi + i + (size_t)w * a.ld);
            if ((unsigned)j >= (unsigned)a.n) {      // e.g. 1-based ids: flagged, not read
                atomicOr(err, 2);
                continue;
            }
            double sx = mi(px - a.x[j], a.len[0], a.half[0], a.ifpd[0]);
            double sy = mi(py - a.y[j], a.len[1], a.half[1], a.ifpd[1]);
            double sz = mi(pz - a.z[j], a.len[2], a.half[2], a.ifpd[2]);
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 <= a.ru2) {
                double sk = sqrt(sqrt(r2)) * a.csi;
                int kk = (int)sk;
                rho += lerp_ref(a.potb, a.ntab, kk, sk - kk);
            }
        }
        if (rho > 0.0) {
            if (a.pottype == MSMGB_FS_TYPE) {
                rho = -0.5 / sqrt(rho);
            } else {
                double sk = rho / a.rhod + 1.0;
                int kk = (int)(sk + 0.000001);
                if (kk + 1 > a.nembd) atomicOr(err, 1);
                rho = lerp_ref(a.dfembd, a.nembd, kk, sk - kk);
            }
        }
    }
    den[i] = rho;
}

__global__ void __launch_bounds__(256) k_na_force(NaArgs a, const double *den, int *err)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if ((a.statu[i] & MSMGB_STATU_ACTIVE) == MSMGB_STATU_ACTIVE) {
        const double px = a.x[i], py = a.y[i], pz = a.z[i];
        const double di = den[i];
        const int kn = a.kvois[i];
        for (int w = 0; w < kn; ++w) {
            int j = __ldg(a.indi + i + (size_t)w * a.ld);
            if ((unsigned)j >= (unsigned)a.n) {
                atomicOr(err, 2);
                continue;
            }
            double sx = mi(px - a.x[j], a.len[0], a.half[0], a.ifpd[0]);
            double sy = mi(py - a.y[j], a.len[1], a.half[1], a.ifpd[1]);
            double sz = mi(pz - a.z[j], a.len[2], a.half[2], a.ifpd[2]);
            double r2 = sx * sx + sy * sy + sz * sz;
            if (r2 <= a.ru2) {
                double r = sqrt(r2);
                double sk = sqrt(r) * a.csi;
                int kk = (int)sk;
                double dk = sk - kk;
                double B = lerp_ref(a.fpotb, a.ntab, kk, dk);
                double ft = lerp_ref(a.fpotr, a.ntab, kk, dk) / r2 + B * (di + den[j]) / r;
                fx += ft * sx;
                fy += ft * sy;
                fz += ft * sz;
            }
        }
    }
    a.fp[i] = fx;
    a.fp[(size_t)a.n + i] = fy;
    a.fp[2 * (size_t)a.n + i] = fz;
}

// once per device, with that device current: device addresses of the file-scope arrays
int scratch_for_current_device(const msmgb_force_noalloc *args, DevScratch **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        put_msg(args, "no usable current CUDA device");
        return MSMGB_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DevScratch &s = g_dev[dev];
    if (!s.ready) {
        void *p = nullptr, *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_den_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_err_scratch);
        if (e != cudaSuccess) {
            char buf[256];
            snprintf(buf, sizeof(buf), "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            put_msg(args, buf);
            return MSMGB_ERR_CUDA;
        }
        s.den = (double *)p;
        s.err = (int *)q;
        s.ready = true;
    }
    *out = &s;
    return MSMGB_OK;
}

}  // namespace

extern "C" int msmgb_calforce_noalloc(const msmgb_force_noalloc *args)
{
    if (!args) return MSMGB_ERR_ARG;
    const msmgb_force_noalloc &a = *args;
    if (a.n < 1 || !a.xp || !a.statu || !a.kvois || !a.indi || !a.potb || !a.fpotr || !a.fpotb ||
        !a.fp || a.ntab < 2 || a.rmax <= 0.0 || a.ld < a.n) {
        put_msg(args, "msmgb_calforce_noalloc: missing array or bad size");
        return MSMGB_ERR_ARG;
    }
    if (a.n > kNoAllocMaxAtoms) {
        char buf[160];
        snprintf(buf, sizeof(buf), "msmgb_calforce_noalloc: %d atoms exceed the fixed scratch of %d atoms "
                 "(MSMGB_NOALLOC_MAX_ATOMS); use a context instead", a.n, kNoAllocMaxAtoms);
        put_msg(args, buf);
        return MSMGB_ERR_CAPACITY;
    }
    if (a.pottype != MSMGB_FS_TYPE && a.pottype != MSMGB_EAM_TYPE) {
        put_msg(args, "msmgb_calforce_noalloc: unknown potential type");
        return MSMGB_ERR_ARG;
    }
    if (a.pottype == MSMGB_EAM_TYPE && (!a.dfembd || a.nembd < 2 || a.rhod <= 0.0)) {
        put_msg(args, "msmgb_calforce_noalloc: EAM needs DFEMBD, NEMBD and RHOD");
        return MSMGB_ERR_ARG;
    }
    DevScratch *s = nullptr;
    int rc = scratch_for_current_device(args, &s);
    if (rc != MSMGB_OK) return rc;
    NaArgs k;
    k.n = a.n;
    k.ld = a.ld;
    k.ntab = a.ntab;
    k.nembd = a.nembd;
    k.pottype = a.pottype;
    k.x = a.xp;
    k.y = a.xp + a.n;
    k.z = a.xp + 2 * (size_t)a.n;
    k.statu = a.statu;
    k.kvois = a.kvois;
    k.indi = a.indi;
    for (int d = 0; d < 3; ++d) {
        k.len[d] = a.box_len[d];
        k.half[d] = 0.5 * a.box_len[d];
        k.ifpd[d] = a.ifpd[d] ? 1 : 0;
    }
    k.csi = (double)a.ntab / sqrt(a.rmax);
    k.ru2 = a.ru * a.ru;
    k.rhod = a.rhod;
    k.potb = a.potb;
    k.fpotr = a.fpotr;
    k.fpotb = a.fpotb;
    k.dfembd = a.dfembd;
    k.fp = a.fp;
    cudaStream_t st = (cudaStream_t)a.stream;
    cudaError_t e = cudaMemsetAsync(s->err, 0, sizeof(int), st);    // error word starts at zero
    int grid = (a.n + 255) / 256;
    if (e == cudaSuccess) {
        k_na_density<<<grid, 256, 0, st>>>(k, s->den, s->err);
        k_na_force<<<grid, 256, 0, st>>>(k, s->den, s->err);
        e = cudaGetLastError();
    }
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "msmgb_calforce_noalloc: CUDA error %s", cudaGetErrorString(e));
        put_msg(args, buf);
        return MSMGB_ERR_CUDA;
    }
    if (herr & 2) {
        put_msg(args, "msmgb_calforce_noalloc: a neighbour id in INDI lies outside 0..n-1 (the ids are "
                      "0-based; a 1-based Fortran list must be converted first); those slots were skipped");
        return MSMGB_ERR_ARG;
    }
    if (herr & 1) {
        put_msg(args, "msmgb_calforce_noalloc: electron density beyond the F(rho) table");
        return MSMGB_ERR_RHO_RANGE;
    }
    return MSMGB_OK;
}
