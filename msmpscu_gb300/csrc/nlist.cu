// nlist.cu -- device cell binning, cell sort and full neighbour list.
//
// Replaces Cal_NeighBoreList2C_0_DEV (MD_NeighborsList_GPU.F90:1347-1732).  The reference
// bins on the device, copies ~10 N-length arrays to the host, builds linked cells there,
// gathers the atoms in cell order, copies them back and then runs one CTA per cell
// (Cal_NeighboreList_Kernel2C, :907-1199).  Here every stage stays on the device:
//   k_bin       cell id per atom (NeighboreList_IC_KERNEL formula, :759-819) + histogram over
//               the cells' storage positions (each box's cells in Morton order of (ix, iy, iz))
//   scan        exclusive scan of the cell histogram (cell start offsets, hm_IA1th)
//   k_scatter   counting-sort scatter, then k_cellsort orders each cell by previous index
//               so the permutation is deterministic
//   k_permute   gathers the atom state into cell order (hm_XP/hm_GID gather, :1541-1570)
//   k_build     one thread per atom scans the 27-cell stencil in the reference's order
//               (own cell first, then NIX/NIY/NIZ, MD_NeighborsList.F90:423-425); an FP32
//               distance test decides every pair outside a narrow band around the cutoff,
//               pairs inside the band get the exact FP64 rule d^2 < rc^2
//               (MD_NeighborsList.F90:605), so the sets equal the FP64 oracle's.  Boxes
//               whose cells are at least rc_nl wide take the image shift of the stencil
//               cell; boxes with NCELL forced to 3 the minimum image of every candidate.
// In an MD-step graph the rebuild is the body of a conditional node that the step's
// decision kernel switches on (context.cu), so steps without a rebuild launch none of these.
#include <algorithm>
#include <climits>

#include "msmgb_internal.cuh"

namespace msmgb {

__constant__ int c_nix[27] = {0, -1, -1, -1, 0, 0, -1, 1, -1, 0, 1, -1, 0, 1, 1, 1, 1, 0, 0, -1, 1, -1, 0, 1, -1, 0, 1};
__constant__ int c_niy[27] = {0, 0, -1, 1, 1, 0, 0, 0, -1, -1, -1, 1, 1, 1, 0, 1, -1, -1, 0, 0, 0, -1, -1, -1, 1, 1, 1};
__constant__ int c_niz[27] = {0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, -1};

__global__ void k_zero_int(int *p, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

// cell index per atom: int((x - lo)/L * NC - 1e-4), MD_NeighborsList_GPU.F90:800-811
__global__ void k_bin(DevAtoms a, int sentinel, int *cell_of, const int *rank, int *count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int st = a.statu[i];
    int c;
    if (st & MSMGB_STATU_OUTOFBOX) {
        c = sentinel;
    } else {
        const DevBox &b = a.box[a.boxid[i]];
        double4_32a p = a.pos[i];
        double xp[3] = {p.x, p.y, p.z};
        if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(&a.flags[kFlagErr], kErrNonFinite);
        int ix[3];
        bool bad = false;
        for (int k = 0; k < 3; ++k) {
            int t = (int)((xp[k] - b.lo[k]) / b.len[k] * (double)b.nc[k] - 0.0001);
            if (t < 0 || t > b.nc[k]) bad = true;
            t = t < 0 ? 0 : (t >= b.nc[k] ? b.nc[k] - 1 : t);
            ix[k] = t;
        }
        if (bad) atomicOr(&a.flags[kFlagErr], kErrOutOfBox);
        c = b.cell0 + ix[0] + b.nc[0] * (ix[1] + b.nc[1] * ix[2]);
    }
    cell_of[i] = c;
    atomicAdd(&count[rank[c]], 1);
}

// ---- exclusive scan (4096 items per block, block sums scanned by one block) ------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int *total)
{
    __shared__ int warp_sums[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    int excl = x - v + (wid > 0 ? warp_sums[wid - 1] : 0);
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const int *in, int *out, int n, int *sums)
{
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int e = block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
    if (threadIdx.x == 0 && sums) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(int *out, int n, const int *sums)
{
    if (blockIdx.x == 0) return;
    int add = sums[blockIdx.x];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) out[base + k] += add;
}

// ---- counting-sort scatter and deterministic per-cell order --------------------------
__global__ void k_scatter(DevAtoms a, const int *cell_of, const int *rank, const int *start, int *cursor, int *perm)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int c = rank[cell_of[i]];
    int slot = start[c] + atomicAdd(&cursor[c], 1);
    perm[slot] = i;
}

__global__ void k_cellsort(int ncs, const int *start, int *perm)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncs) return;
    int b = start[c], e = start[c + 1];
    for (int i = b + 1; i < e; ++i) {   // insertion sort: cells hold ~10 atoms
        int v = perm[i];
        int j = i - 1;
        while (j >= b && perm[j] > v) { perm[j + 1] = perm[j]; --j; }
        perm[j + 1] = v;
    }
}

// staging layout inside the scratch buffer (one slab per field, capacity entries each)
struct Stage {
    double4_32a *pos;
    double *vx, *vy, *vz, *dx, *dy, *dz;
    int *ityp, *statu, *gid, *boxid, *cell;
};

__host__ __device__ inline Stage stage_of(void *scratch, int cap)
{
    Stage s;
    char *p = (char *)scratch;
    s.pos = (double4_32a *)p; p += sizeof(double4_32a) * (size_t)cap;
    s.vx = (double *)p; p += sizeof(double) * (size_t)cap;
    s.vy = (double *)p; p += sizeof(double) * (size_t)cap;
    s.vz = (double *)p; p += sizeof(double) * (size_t)cap;
    s.dx = (double *)p; p += sizeof(double) * (size_t)cap;
    s.dy = (double *)p; p += sizeof(double) * (size_t)cap;
    s.dz = (double *)p; p += sizeof(double) * (size_t)cap;
    s.ityp = (int *)p; p += sizeof(int) * (size_t)cap;
    s.statu = (int *)p; p += sizeof(int) * (size_t)cap;
    s.gid = (int *)p; p += sizeof(int) * (size_t)cap;
    s.boxid = (int *)p; p += sizeof(int) * (size_t)cap;
    s.cell = (int *)p;
    return s;
}

__global__ void k_permute(DevAtoms a, Stage s, const int *perm, const int *cell_of)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int o = perm[i];
    s.pos[i] = a.pos[o];
    s.vx[i] = a.vx[o]; s.vy[i] = a.vy[o]; s.vz[i] = a.vz[o];
    s.dx[i] = a.dx[o]; s.dy[i] = a.dy[o]; s.dz[i] = a.dz[o];
    s.ityp[i] = a.ityp[o];
    s.statu[i] = a.statu[o];
    s.gid[i] = a.gid[o];
    s.boxid[i] = a.boxid[o];
    s.cell[i] = cell_of[o];
}

__global__ void k_copyback(DevAtoms a, Stage s, int *cell_of)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double4_32a p = s.pos[i];
    a.pos[i] = p;
    const PosFF f = make_posff(p.x, p.y, p.z, a.box[s.boxid[i]]);
    a.posff[i] = f;
    a.pos_bld[i] = pos_f32(f);   // skin reference and k_build candidates
    a.vx[i] = s.vx[i]; a.vy[i] = s.vy[i]; a.vz[i] = s.vz[i];
    a.dx[i] = s.dx[i]; a.dy[i] = s.dy[i]; a.dz[i] = s.dz[i];
    a.ityp[i] = s.ityp[i];
    a.statu[i] = s.statu[i];
    a.gid[i] = s.gid[i];
    a.boxid[i] = s.boxid[i];
    cell_of[i] = s.cell[i];
}

__device__ __forceinline__ double mi64(double s, double len, double half, int pd)
{
    return (pd && fabs(s) > half) ? s - copysign(len, s) : s;
}

__device__ __forceinline__ float mi32(float s, float len, float half, int pd)
{
    return (pd && fabsf(s) > half) ? s - copysignf(len, s) : s;
}

// The exact FP64 rule of the oracle: d^2 < rc^2 on the FP64 positions after the minimum image.
__device__ __forceinline__ bool fp64_rule(const DevAtoms &a, int i, int j, const DevBox &b, double rc2)
{
    const double4_32a p = a.pos[i];
    const double4_32a qd = a.pos[j];
    const double dx = mi64(p.x - qd.x, b.len[0], b.half[0], b.ifpd[0]);
    const double dy = mi64(p.y - qd.y, b.len[1], b.half[1], b.ifpd[1]);
    const double dz = mi64(p.z - qd.z, b.len[2], b.half[2], b.ifpd[2]);
    return (dx * dx + dy * dy + dz * dz) < rc2;
}

// Records a candidate that passed the FP32 test or, inside the narrow band around the
// cutoff, the exact FP64 rule.
__device__ __forceinline__ bool accept(float d2f, float d2lo, float d2hi, const DevAtoms &a, int i, int j,
                                       const DevBox &b, double rc2)
{
    if (d2f < d2lo) return true;
    if (d2f > d2hi) return false;
    return fp64_rule(a, i, j, b, rc2);
}

// Full neighbour list, one thread per (sorted) atom.  Cells of a box are at least rc_nl
// wide unless the box forced NCELL to 3 (the reference's rule for small boxes); in the wide
// case the periodic image of every candidate is the one of its stencil cell, so the
// separation is the exact difference of the FP32 positions plus a per-cell shift of -L, 0 or +L, with no
// per-candidate minimum-image test.  Narrow boxes take the minimum image per candidate.
__global__ void __launch_bounds__(kBlock, 6) k_build(DevAtoms a, const int *cell_of, const int *rank,
                                                  const int *start, double rc2, float d2lo, float d2hi)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 pf = pos_f32(a.posff[i]);
    if (a.statu[i] & MSMGB_STATU_OUTOFBOX) { a.kvois[i] = 0; return; }
    const DevBox &b = a.box[a.boxid[i]];
    int nc[3], pd[3];
    float lf[3];
    bool wide = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nc[k] = b.nc[k];
        pd[k] = b.ifpd[k];
        lf[k] = b.lenf[k];
        const double w = b.len[k] / nc[k];
        if (pd[k] && w * w < rc2) wide = false;
    }
    const int cell0 = b.cell0;
    const int c = cell_of[i] - cell0;
    const int ix = c % nc[0], iy = (c / nc[0]) % nc[1], iz = c / (nc[0] * nc[1]);
    int nn = 0;
    const size_t ld = (size_t)a.ld;
    const int mxk = a.mxk;
    int *const indi = a.indi + i;
    const float4 *const hi = a.pos_bld;   // FP32 positions, 16 B per atom (written by k_copyback)
    for (int s = 0; s < 27; ++s) {
        int j3[3] = {ix + c_nix[s], iy + c_niy[s], iz + c_niz[s]};
        float sh[3];
        bool skip = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sh[k] = 0.0f;
            if (pd[k]) {
                // candidate cell wrapped to the other end: its image lies one box length away
                if (j3[k] >= nc[k]) { j3[k] = 0; sh[k] = -lf[k]; }
                else if (j3[k] < 0) { j3[k] = nc[k] - 1; sh[k] = lf[k]; }
            }
            if (j3[k] < 0 || j3[k] >= nc[k]) skip = true;
        }
        if (skip) continue;
        const int g = rank[cell0 + j3[0] + nc[0] * (j3[1] + nc[1] * j3[2])];
        const int j0 = start[g], e = start[g + 1];
        if (wide) {
            for (int j = j0; j < e; ++j) {
                const float4 q = hi[j];
                const float sx = (pf.x - q.x) + sh[0];       // difference exact (Sterbenz)
                const float sy = (pf.y - q.y) + sh[1];
                const float sz = (pf.z - q.z) + sh[2];
                const float d2f = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
                if (j != i && accept(d2f, d2lo, d2hi, a, i, j, b, rc2)) {
                    if (nn < mxk) indi[(size_t)nn * ld] = j;
                    ++nn;
                }
            }
        } else {
            const float h0 = b.halff[0], h1 = b.halff[1], h2 = b.halff[2];
            for (int j = j0; j < e; ++j) {
                const float4 q = hi[j];
                const float sx = mi32(pf.x - q.x, lf[0], h0, pd[0]);
                const float sy = mi32(pf.y - q.y, lf[1], h1, pd[1]);
                const float sz = mi32(pf.z - q.z, lf[2], h2, pd[2]);
                const float d2f = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
                if (j != i && accept(d2f, d2lo, d2hi, a, i, j, b, rc2)) {
                    if (nn < mxk) indi[(size_t)nn * ld] = j;
                    ++nn;
                }
            }
        }
    }
    if (nn > mxk) {
        atomicOr(&a.flags[kFlagErr], kErrOverflow);
        nn = mxk;
    }
    a.kvois[i] = nn;
    atomicMax(&a.flags[kFlagMaxK], nn);
}

// A state with a non-cubic box: every candidate by the FP64 rule on BOXSHAPE . SEP (cubic
// boxes of the same state take the same path); cells were sized so that the stencil covers
// rc_nl after the shape.  No two-level list.
__global__ void __launch_bounds__(kBlock) k_build_shaped(DevAtoms a, const int *cell_of, const int *rank,
                                                         const int *start, double rc2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if (a.statu[i] & MSMGB_STATU_OUTOFBOX) { a.kvois[i] = 0; return; }
    const DevBox &b = a.box[a.boxid[i]];
    int nc[3], pd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nc[k] = b.nc[k];
        pd[k] = b.ifpd[k];
    }
    const int cell0 = b.cell0;
    const int c = cell_of[i] - cell0;
    const int ix = c % nc[0], iy = (c / nc[0]) % nc[1], iz = c / (nc[0] * nc[1]);
    int nn = 0;
    const size_t ld = (size_t)a.ld;
    const int mxk = a.mxk;
    int *const indi = a.indi + i;
    const double4_32a p = a.pos[i];
    for (int s = 0; s < 27; ++s) {
        int j3[3] = {ix + c_nix[s], iy + c_niy[s], iz + c_niz[s]};
        bool skip = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (pd[k]) j3[k] = (j3[k] + nc[k]) % nc[k];
            else if (j3[k] < 0 || j3[k] >= nc[k]) skip = true;
        }
        if (skip) continue;
        const int g = rank[cell0 + j3[0] + nc[0] * (j3[1] + nc[1] * j3[2])];
        const int j0 = start[g], e = start[g + 1];
        for (int j = j0; j < e; ++j) {
            const double4_32a q = a.pos[j];
            double dx = mi64(p.x - q.x, b.len[0], b.half[0], b.ifpd[0]);
            double dy = mi64(p.y - q.y, b.len[1], b.half[1], b.ifpd[1]);
            double dz = mi64(p.z - q.z, b.len[2], b.half[2], b.ifpd[2]);
            shape_sep(b, dx, dy, dz);
            if (j != i && dx * dx + dy * dy + dz * dz < rc2) {
                if (nn < mxk) indi[(size_t)nn * ld] = j;
                ++nn;
            }
        }
    }
    if (nn > mxk) {
        atomicOr(&a.flags[kFlagErr], kErrOverflow);
        nn = mxk;
    }
    a.kvois[i] = nn;
    atomicMax(&a.flags[kFlagMaxK], nn);
}

// ---- two-level list -----------------------------------------------------------------------
// With an outer skin s_o > 0 a full rebuild (binning, sort, permutation) stores, per atom, the
// candidates within rc_nl + s_o (k_build_cand, FP32 test with the prefilter margin: a superset
// of the pairs whose exact distance is below rc_nl + s_o), and every list build, full or not,
// selects from those candidates the pairs with d^2 < rc_nl^2 by the same FP32 prefilter and
// FP64 band rule as k_build (k_inner).  Between full rebuilds no atom moves more than s_o / 2
// (k_decide bounds the displacement since the full rebuild by the sum of the skin maxima of
// the rebuild intervals), so a pair within rc_nl now was within rc_nl + s_o then and the
// lists are the sets k_build would give.  The atoms keep their cell order between full
// rebuilds.
__global__ void __launch_bounds__(kBlock, 6) k_build_cand(DevAtoms a, const int *cell_of, const int *rank,
                                                       const int *start, int *cand, int *kcand, int mxo, float d2o,
                                                       double ro2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {                          // displacement bound and box exits since this full rebuild
        a.flags[kFlagAcc] = 0;
        a.flags[kFlagOob] = 0;
    }
    // (kFlagMaxCand is cleared by the host before a build it checks)
    if (i >= a.n) return;
    if (a.statu[i] & MSMGB_STATU_OUTOFBOX) { kcand[i] = 0; return; }
    const float4 pf = a.pos_bld[i];
    const DevBox &b = a.box[a.boxid[i]];
    int nc[3], pd[3];
    float lf[3], hf[3];
    bool wide = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nc[k] = b.nc[k];
        pd[k] = b.ifpd[k];
        lf[k] = b.lenf[k];
        hf[k] = b.halff[k];
        const double w = b.len[k] / nc[k];
        if (pd[k] && w * w < ro2) wide = false;
    }
    const int cell0 = b.cell0;
    const int c = cell_of[i] - cell0;
    const int ix = c % nc[0], iy = (c / nc[0]) % nc[1], iz = c / (nc[0] * nc[1]);
    int nn = 0;
    const size_t ld = (size_t)a.ld;
    int *__restrict__ const out = cand + i;
    const float4 *__restrict__ const hi = a.pos_bld;
    for (int s = 0; s < 27; ++s) {
        int j3[3] = {ix + c_nix[s], iy + c_niy[s], iz + c_niz[s]};
        float sh[3];
        bool skip = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sh[k] = 0.0f;
            if (pd[k]) {
                // candidate cell wrapped to the other end: its image lies one box length away
                if (j3[k] >= nc[k]) { j3[k] = 0; sh[k] = -lf[k]; }
                else if (j3[k] < 0) { j3[k] = nc[k] - 1; sh[k] = lf[k]; }
            }
            if (j3[k] < 0 || j3[k] >= nc[k]) skip = true;
        }
        if (skip) continue;
        const int g = rank[cell0 + j3[0] + nc[0] * (j3[1] + nc[1] * j3[2])];
        const int j0 = start[g], e = start[g + 1];
        if (wide) {   // cells of at least rc_nl + skin: the stencil cell's image is the nearest
            // atom i's position shifted once per stencil cell (the shift's rounding, at most
            // ulp(3L)/2 per component, lies inside the prefilter margin of this superset test);
            // unrolled over restrict pointers: 2.544 against 2.570 ms per full rebuild of the
            // 2,048,000-atom Cu state
            const float px = pf.x + sh[0], py = pf.y + sh[1], pz = pf.z + sh[2];
#pragma unroll 4
            for (int j = j0; j < e; ++j) {
                const float4 q = __ldg(hi + j);
                const float sx = px - q.x;
                const float sy = py - q.y;
                const float sz = pz - q.z;
                const float d2f = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
                if (j != i && d2f < d2o) {
                    if (nn < mxo) out[(size_t)nn * ld] = j;
                    ++nn;
                }
            }
        } else {
            for (int j = j0; j < e; ++j) {
                const float4 q = hi[j];
                const float sx = mi32(pf.x - q.x, lf[0], hf[0], pd[0]);
                const float sy = mi32(pf.y - q.y, lf[1], hf[1], pd[1]);
                const float sz = mi32(pf.z - q.z, lf[2], hf[2], pd[2]);
                const float d2f = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
                if (j != i && d2f < d2o) {
                    if (nn < mxo) out[(size_t)nn * ld] = j;
                    ++nn;
                }
            }
        }
    }
    atomicMax(&a.flags[kFlagMaxCand], nn);
    if (nn > mxo) {
        atomicOr(&a.flags[kFlagErr], kErrCandOverflow);
        nn = mxo;
    }
    kcand[i] = nn;
}

// accept() for a candidate whose float-float record pj is at hand: inside the FP32 band, the
// float-float distance of the two records (hi parts on the quantum, so the sum of squared hi
// differences is exact; the lo parts as dl (2 dh + dl)) lies within ~5e-8 A^2 of the FP64 one
// (lo parts within (2^-26 + 2^-33) of the quantum, the rounding of the lo terms), so the FP64 rule
// decides only pairs within 2e-7 A^2 of rc^2: the same sets, with the FP64 pipe nearly idle.
// The sum of squared hi differences is exact below 2^24 quanta^2 (rc below 32 A at the smallest
// quantum); beyond that the caller passes rc2h < 0 and every band pair takes the FP64 rule.
__device__ __forceinline__ bool accept_ff(float d2f, float d2lo, float d2hi, const DevAtoms &a, int i, int j,
                                          const PosFF &pj, const DevBox &b, double rc2, float rc2h, float rc2l)
{
    if (d2f < d2lo) return true;
    if (d2f > d2hi) return false;
    if (rc2h < 0.0f) return fp64_rule(a, i, j, b, rc2);
    const PosFF pi = ld_ff(a.posff + i);
    const float hi[3] = {pi.hx, pi.hy, pi.hz}, li[3] = {pi.lx, pi.ly, pi.lz};
    const float hj[3] = {pj.hx, pj.hy, pj.hz}, lj[3] = {pj.lx, pj.ly, pj.lz};
    float S = 0.0f, C = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float dh = hi[k] - hj[k];                      // exact multiple of the quantum
        float dl = li[k] - lj[k];
        if (b.ifpd[k] && fabsf(dh) > b.halff[k]) {
            const float sg = copysignf(1.0f, dh);
            dh = fmaf(-sg, b.fixlq[k], dh);            // exact (L rounded to the quantum)
            dl = fmaf(-sg, b.fixll[k], dl);
        }
        S = fmaf(dh, dh, S);                           // exact
        C = fmaf(dl, fmaf(2.0f, dh, dl), C);
    }
    const float diff = (S - rc2h) + (C - rc2l);        // S - rc2h exact (Sterbenz)
    if (diff < -2e-7f) return true;
    if (diff > 2e-7f) return false;
    return fp64_rule(a, i, j, b, rc2);
}

// The list from the candidates at the current positions; also the skin reference pos_bld.
// Candidates are taken kInnerUnr at a time, their indices one group ahead, so the position
// gathers of a group overlap.  No candidate has left its box: an exit since the full rebuild
// makes the next rebuild full (kFlagOob).
constexpr int kInnerUnr = 4;

__global__ void __launch_bounds__(kBlock, 4) k_inner(DevAtoms a, const int *cand, const int *kcand, double rc2,
                                                  float d2lo, float d2hi, float rc2h, float rc2l)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 pf = pos_f32(a.posff[i]);
    a.pos_bld[i] = pf;
    if (!(isfinite(pf.x) && isfinite(pf.y) && isfinite(pf.z))) atomicOr(&a.flags[kFlagErr], kErrNonFinite);
    // an atom outside its box neither has nor is a neighbour (the full rebuild puts it into
    // the sentinel cell)
    if (a.statu[i] & MSMGB_STATU_OUTOFBOX) { a.kvois[i] = 0; return; }
    const int kc = kcand[i];
    const DevBox &b = a.box[a.boxid[i]];
    float lf[3], hf[3];
    int pd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lf[k] = b.lenf[k];
        hf[k] = b.halff[k];
        pd[k] = b.ifpd[k];
    }
    const size_t ld = (size_t)a.ld;
    const int mxk = a.mxk;
    int *const indi = a.indi + i;
    const int *const cd = cand + i;
    int nn = 0;
    int jn[kInnerUnr];
#pragma unroll
    for (int u = 0; u < kInnerUnr; ++u) jn[u] = u < kc ? __ldg(cd + (size_t)u * ld) : i;
    for (int s = 0; s < kc; s += kInnerUnr) {
        int j[kInnerUnr];
        PosFF q[kInnerUnr];
#pragma unroll
        for (int u = 0; u < kInnerUnr; ++u) {
            j[u] = jn[u];
            const int sl = s + kInnerUnr + u;
            jn[u] = sl < kc ? __ldg(cd + (size_t)sl * ld) : i;
        }
#pragma unroll
        for (int u = 0; u < kInnerUnr; ++u) q[u] = ld_ff(a.posff + j[u]);   // one 256-bit load
#pragma unroll
        for (int u = 0; u < kInnerUnr; ++u) {
            if (s + u >= kc) break;
            const float4 g = pos_f32(q[u]);
            const float sx = mi32(pf.x - g.x, lf[0], hf[0], pd[0]);
            const float sy = mi32(pf.y - g.y, lf[1], hf[1], pd[1]);
            const float sz = mi32(pf.z - g.z, lf[2], hf[2], pd[2]);
            const float d2f = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
            if (accept_ff(d2f, d2lo, d2hi, a, i, j[u], q[u], b, rc2, rc2h, rc2l)) {
                if (nn < mxk) indi[(size_t)nn * ld] = j[u];
                ++nn;
            }
        }
    }
    if (nn > mxk) {
        atomicOr(&a.flags[kFlagErr], kErrOverflow);
        nn = mxk;
    }
    a.kvois[i] = nn;
    atomicMax(&a.flags[kFlagMaxK], nn);
}

// Debug validation of a freshly built list (no trap): every stored neighbour index lies in
// [0, n), differs from the atom itself and belongs to the same box; KVOIS lies in [0, MXKVOIS].
__global__ void k_check_list(DevAtoms a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int m = a.kvois[i];
    bool bad = m < 0 || m > a.mxk;
    const int mm = bad ? 0 : m;
    const size_t ld = (size_t)a.ld;
    for (int k = 0; k < mm && !bad; ++k) {
        const int j = a.indi[(size_t)k * ld + i];
        bad = j < 0 || j >= a.n || j == i || a.boxid[j] != a.boxid[i];
    }
    if (bad) atomicOr(&a.flags[kFlagErr], kErrBadList);
}

// ---- cell tiles of the mixed passes -------------------------------------------------------
// One block per kBlock sorted atoms (the blocks of the pass kernels).  Atoms are sorted by
// cell storage position, so the block's atoms fill the cells of one range of storage
// positions [r0, r1]; the halo is the union of the 27-cell stencils of those cells.  The
// candidate cells are sorted and merged into runs of consecutive storage positions, which
// are runs of consecutive atoms: the pass kernels stage a run with coalesced loads.  Each
// list slot is then translated to its neighbour's position in the staged halo (a binary
// search over the runs), so the passes gather neighbours from shared memory.
constexpr int kHaloCand = 2048;   // >= 27 * kHaloCells, a power of two (bitonic sort)
static_assert(kHaloCand >= 27 * kHaloCells, "candidate buffer");

__global__ void __launch_bounds__(kBlock) k_halo(DevAtoms a, const int *cell_of, const int *rank, const int *unrank,
                                                 const int *start, int sentinel)
{
    __shared__ int cand[kHaloCand];
    __shared__ int r_first[kHaloRuns + 1], r_soff[kHaloRuns + 1], r_end[kHaloRuns];
    __shared__ int s_cnt[kBlock];
    __shared__ int s_bad, s_nrun;
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * kBlock;
    const int n = a.n;
    const int i1 = min(i0 + kBlock, n) - 1;
    const int r0 = rank[cell_of[i0]], r1 = rank[cell_of[i1]];
    const int ncell = r1 - r0 + 1;
    if (t == 0) s_bad = ncell > kHaloCells;
    for (int k = t; k < kHaloCand; k += kBlock) cand[k] = INT_MAX;
    __syncthreads();
    if (!s_bad) {
        for (int q = t; q < 27 * ncell; q += kBlock) {
            const int r = r0 + q / 27, s = q % 27;
            if (r == sentinel) continue;                 // out-of-box atoms have no neighbours
            const int a0 = start[r];
            if (start[r + 1] == a0) continue;            // no atom of the block in this cell
            const DevBox &b = a.box[a.boxid[a0]];
            const int l = unrank[r] - b.cell0;
            int j3[3] = {l % b.nc[0] + c_nix[s], (l / b.nc[0]) % b.nc[1] + c_niy[s], l / (b.nc[0] * b.nc[1]) + c_niz[s]};
            bool skip = false;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (b.ifpd[k]) j3[k] = (j3[k] + b.nc[k]) % b.nc[k];
                else if (j3[k] < 0 || j3[k] >= b.nc[k]) skip = true;
            }
            if (!skip) cand[q] = rank[b.cell0 + j3[0] + b.nc[0] * (j3[1] + b.nc[1] * j3[2])];
        }
    }
    __syncthreads();
    if (s_bad) {
        if (t == 0) a.hmeta[blockIdx.x] = make_int2(-1, 0);
        return;
    }
    // bitonic sort of the candidate storage positions (ascending; INT_MAX pads)
    for (int k = 2; k <= kHaloCand; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int x = t; x < kHaloCand; x += kBlock) {
                const int y = x ^ j;
                if (y > x) {
                    const int u = cand[x], v = cand[y];
                    if ((u > v) == ((x & k) == 0)) { cand[x] = v; cand[y] = u; }
                }
            }
            __syncthreads();
        }
    }
    // runs: maximal sequences of storage positions with steps of 0 or 1
    constexpr int kPer = kHaloCand / kBlock;
    const int x0 = t * kPer;
    int heads = 0;
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int x = x0 + m, v = cand[x];
        if (v != INT_MAX && (x == 0 || (cand[x - 1] != v && cand[x - 1] != v - 1))) ++heads;
    }
    s_cnt[t] = heads;
    __syncthreads();
    if (t == 0) {
        int acc = 0;
        for (int k = 0; k < kBlock; ++k) { const int h = s_cnt[k]; s_cnt[k] = acc; acc += h; }
        s_nrun = acc;
        if (acc > kHaloRuns) s_bad = 1;
    }
    __syncthreads();
    const int nrun = s_nrun;
    if (!s_bad) {
        int id = s_cnt[t] - 1;
#pragma unroll
        for (int m = 0; m < kPer; ++m) {
            const int x = x0 + m, v = cand[x];
            if (v == INT_MAX) break;
            if (x == 0 || (cand[x - 1] != v && cand[x - 1] != v - 1)) r_first[++id] = start[v];
            const int w = x + 1 < kHaloCand ? cand[x + 1] : INT_MAX;
            if (w != v && w != v + 1) r_end[id] = start[v + 1];
        }
    }
    __syncthreads();
    if (t == 0 && !s_bad) {
        int acc = 0;
        for (int r = 0; r < nrun; ++r) { r_soff[r] = acc; acc += r_end[r] - r_first[r]; }
        r_soff[nrun] = acc;
        if (acc > kHaloMax) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) {
        if (t == 0) a.hmeta[blockIdx.x] = make_int2(-1, 0);
        return;
    }
    // list slots -> halo positions
    const int i = i0 + t;
    if (i < n) {
        const int kn = a.kvois[i];
        const size_t ld = (size_t)a.ld;
        bool miss = false;
        for (int sl = 0; sl < kn; ++sl) {
            const int j = a.indi[(size_t)sl * ld + i];
            int lo = 0, hi = nrun - 1;          // last run whose first atom is <= j
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (r_first[mid] <= j) lo = mid;
                else hi = mid - 1;
            }
            const int off = j - r_first[lo];
            if (off < 0 || off >= r_soff[lo + 1] - r_soff[lo]) { miss = true; break; }
            a.lidx[(size_t)sl * ld + i] = (unsigned short)(r_soff[lo] + off);
        }
        if (miss) s_bad = 1;                    // a neighbour outside the stencil cells: no tile
    }
    __syncthreads();
    int2 *runs = a.hruns + (size_t)blockIdx.x * (kHaloRuns + 1);
    for (int r = t; r <= nrun; r += kBlock) runs[r] = make_int2(r < nrun ? r_first[r] : 0, r_soff[r]);
    if (t == 0) a.hmeta[blockIdx.x] = s_bad ? make_int2(-1, 0) : make_int2(nrun, r_soff[nrun]);
}

static inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

int build_halo(msmgb_ctx *c)
{
    if (c->n <= 0) return MSMGB_OK;
    k_halo<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a, c->cell_of, c->cell_rank, c->cell_unrank,
                                                         c->cell_start, c->ncell_total);
    c->launches += 1;
    return check_launch(c, "cell tiles");
}

int enable_halo(msmgb_ctx *c)
{
    if (!c->a.lidx) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        const size_t nb = (size_t)c->a.ld / kBlock;
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->a.lidx, sizeof(unsigned short) * (size_t)c->a.ld * c->a.mxk);
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->a.hmeta, sizeof(int2) * nb);
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->a.hruns, sizeof(int2) * nb * (kHaloRuns + 1));
        if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc cell tiles");
    }
    if (!c->halo_on) {
        c->halo_on = true;
        if (c->list_valid) return build_halo(c);
    }
    return MSMGB_OK;
}

// Margin of the FP32 prefilter: it uses the FP32 positions hi + lo of the shifted coordinates
// (u in [L, 2L], each within ~ulp(u)/2 of u): their difference and the image shift by float(L)
// are exact (Sterbenz), so a separation component is off by at most ulp(2L) +
// |L - float(L)| <= 1.5 ulp(2L); the band below allows 4 ulp of the largest coordinate extent
// plus the rounding of d^2.
static void prefilter_band(const msmgb_ctx *c, double rc2, float *lo, float *hi)
{
    double ext = 1.0;
    for (const DevBox &b : c->hbox)
        for (int k = 0; k < 3; ++k) ext = fmax(ext, fabs(b.lo[k]) + 2.0 * b.len[k]);
    double ulp = ldexp(1.0, ilogb(ext) - 23);
    double delta = 4.0 * ulp;
    double rc = sqrt(rc2);
    double m = 3.0 * (2.0 * rc * delta + delta * delta) + 4.0 * ldexp(rc2, -23);
    m *= 4.0;  // safety factor
    *lo = (float)(rc2 - m);
    *hi = (float)(rc2 + m);
}

bool two_level(const msmgb_ctx *c)
{
    return c->outer_skin > 0.0 && c->bin_rc >= c->p.rc_nl + c->outer_skin && !c->any_shaped;
}

static int ensure_candidates(msmgb_ctx *c, int need = 0)
{
    // slots: MXKVOIS scaled by the volume ratio, at most twice the count the densest box
    // gives for a sphere of rc_nl + skin (+32), so that a large MXKVOIS costs no memory
    const double ro = c->p.rc_nl + c->outer_skin;
    const double r = ro / c->p.rc_nl;
    double by_mxk = ceil(c->p.mxkvois * r * r * r * 1.1);
    double by_rho = 2.0 * (4.0 / 3.0) * 3.14159265358979 * ro * ro * ro * c->max_density + 32.0;
    int mxo = (((int)std::min(by_mxk, by_rho) + 7) / 8) * 8;
    mxo = std::max(mxo, std::max(need, c->mxo));      // never shrinks below a measured need
    if (c->cand && c->mxo == mxo) return MSMGB_OK;
    // allocated by the host-side full build that precedes every step-graph capture
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone)
        return set_err(c, MSMGB_ERR_ARG, "candidate list allocation inside a graph capture");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (c->cand) cudaFree(c->cand);
    if (c->kcand) cudaFree(c->kcand);
    c->cand = c->kcand = nullptr;
    c->mxo = 0;
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->cand, sizeof(int) * (size_t)c->a.ld * (size_t)mxo);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->kcand, sizeof(int) * (size_t)c->a.ld);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc candidate list");
    c->mxo = mxo;
    return MSMGB_OK;
}

int build_full(msmgb_ctx *c)
{
    const int n = c->n;
    const int ncs = c->ncell_total + 1;   // + sentinel cell for out-of-box atoms
    int *count = c->cell_cursor;          // histogram, then re-zeroed as scatter cursor
    cudaStream_t s = c->stream;
    DevAtoms a = c->a;
    const bool two = two_level(c);
    if (two) {
        const int rc = ensure_candidates(c);
        if (rc) return rc;
    }

    k_zero_int<<<nblk(ncs + 1, kBlock), kBlock, 0, s>>>(count, ncs + 1);
    k_bin<<<nblk(n, kBlock), kBlock, 0, s>>>(a, c->ncell_total, c->cell_of, c->cell_rank, count);
    // exclusive scan over ncs + 1 entries: start[ncs] = n
    int ntile = nblk(ncs + 1, kScanTile);
    k_scan_tile<<<ntile, kScanThreads, 0, s>>>(count, c->cell_start, ncs + 1, c->scan_tmp);
    c->launches += 3;
    if (ntile > 1) {
        k_scan_tile<<<1, kScanThreads, 0, s>>>(c->scan_tmp, c->scan_tmp, ntile, nullptr);
        k_scan_add<<<ntile, kScanThreads, 0, s>>>(c->cell_start, ncs + 1, c->scan_tmp);
        c->launches += 2;
    }
    k_zero_int<<<nblk(ncs + 1, kBlock), kBlock, 0, s>>>(count, ncs + 1);
    k_scatter<<<nblk(n, kBlock), kBlock, 0, s>>>(a, c->cell_of, c->cell_rank, c->cell_start, count, c->perm);
    k_cellsort<<<nblk(ncs, kBlock), kBlock, 0, s>>>(ncs, c->cell_start, c->perm);
    Stage st = stage_of(c->scratch, c->cap_atoms);
    k_permute<<<nblk(n, kBlock), kBlock, 0, s>>>(a, st, c->perm, c->cell_of);
    k_copyback<<<nblk(n, kBlock), kBlock, 0, s>>>(a, st, c->cell_of);
    c->launches += 5;
    if (two) {
        const double ro = c->p.rc_nl + c->outer_skin;
        float d2lo, d2hi;
        prefilter_band(c, ro * ro, &d2lo, &d2hi);
        k_build_cand<<<nblk(n, kBlock), kBlock, 0, s>>>(a, c->cell_of, c->cell_rank, c->cell_start, c->cand,
                                                        c->kcand, c->mxo, d2hi, ro * ro);
    } else if (c->any_shaped) {
        k_build_shaped<<<nblk(n, kBlock), kBlock, 0, s>>>(a, c->cell_of, c->cell_rank, c->cell_start,
                                                          c->p.rc_nl * c->p.rc_nl);
    } else {
        double rc2 = c->p.rc_nl * c->p.rc_nl;
        float d2lo, d2hi;
        prefilter_band(c, rc2, &d2lo, &d2hi);
        k_build<<<nblk(n, kBlock), kBlock, 0, s>>>(a, c->cell_of, c->cell_rank, c->cell_start, rc2, d2lo, d2hi);
    }
    c->launches += 1;
    return check_launch(c, "neighbour list");
}

static int finish_list(msmgb_ctx *c)
{
    if (c->check_lists) {
        k_check_list<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a);
        c->launches += 1;
    }
    const int rc = check_launch(c, "neighbour list");
    if (rc || !c->halo_on) return rc;
    return build_halo(c);
}

int build_inner(msmgb_ctx *c)
{
    const double rc2 = c->p.rc_nl * c->p.rc_nl;
    float d2lo, d2hi;
    prefilter_band(c, rc2, &d2lo, &d2hi);
    float rc2h = (float)rc2, rc2l = (float)(rc2 - (double)rc2h);
    {   // the band's float-float decision needs exact sums of squared hi differences (d2hi is
        // the band's upper edge)
        const double q = c->hbox.empty() ? 0.0 : (double)c->hbox[0].qq;
        if (!((double)d2hi < 0.9 * 16777216.0 * q * q)) rc2h = -1.0f;
    }
    k_inner<<<nblk(c->n, kBlock), kBlock, 0, c->stream>>>(c->a, c->cand, c->kcand, rc2, d2lo, d2hi, rc2h, rc2l);
    c->launches += 1;
    return finish_list(c);
}

// Host-side full build.  With a two-level list the largest candidate count is read back: a
// candidate buffer that was too small (a denser region than the boxes' mean density) is
// grown to 1.25 x that count + 16 and the build repeated, and the step graphs, which hold
// the buffer's size, are recaptured.
int build_list(msmgb_ctx *c)
{
    if (!two_level(c)) {
        const int rc = build_full(c);
        return rc ? rc : finish_list(c);
    }
    for (int attempt = 0; attempt < 2; ++attempt) {
        cudaError_t e = cudaMemsetAsync(c->a.flags + kFlagMaxCand, 0, sizeof(int), c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "flag clear");
        int rc = build_full(c);
        if (rc) return rc;
        int got[2] = {0, 0};     // error bits, largest candidate count
        e = cudaMemcpyAsync(&got[0], c->a.flags + kFlagErr, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&got[1], c->a.flags + kFlagMaxCand, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "flag read");
        if (got[1] <= c->mxo) break;
        const int clear = got[0] & ~kErrCandOverflow;
        e = cudaMemcpyAsync(c->a.flags + kFlagErr, &clear, sizeof(int), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "flag clear");
        rc = ensure_candidates(c, (int)(1.25 * got[1]) + 16);
        if (rc) return rc;
        c->graphs_stale = true;
    }
    return build_inner(c);
}

}  // namespace msmgb
