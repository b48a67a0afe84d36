// Throughput mode of the propagation kernel.
//
// Same algorithm as propagate_one<EXACT> (src/integrator.h:648-824 with the
// fused src/lensing.h:399-472 Jacobian), reorganised for the GB300's
// arithmetic balance:
//
//  * Stencil records.  Every cell carries, in HBM, its 27 same-level
//    neighbours resolved with the reference's lookup semantics, a mask of the
//    ones at exactly its level and its level / children flags (built on the
//    GPU at upload, mpf_octree.cu).  A TSC or CIC gather is then one 128-byte
//    record load plus the payload loads; a restart at a coarser neighbour
//    (simplehyperoctree.h:1532-1537) re-centres on the coarser cell's record.
//    The deepest cell of a point near a known cell is read from that cell's
//    record, so the RK stages, the post-step gather and the six Jacobian
//    gathers of a step do no octree walks in the common case.
//  * FP64 is kept for the RK4 state, the RHS, the affine parameter, redshift
//    and distances.  Cell coordinates use exact power-of-two scalings (no
//    divisions), TSC weights and field accumulation are FP32, the cosmology
//    search uses a uniform index table.
#pragma once
#include "mpf_propagate.cuh"

namespace mpf {

constexpr unsigned kFullMask = (1u << 27) - 1u;

// Launch shape of the persistent kernel: threads per block and the minimum
// resident blocks per SM promised to the register allocator.  128 x 2 (up to
// 255 registers, 8 warps per SM) measured fastest on the AMR and medium
// octrees, ahead of 128 x 3 (168 registers, spills) and 128 x 4.
// Overridable at build time for tuning sweeps.
#ifndef MPF_FAST_THREADS
#define MPF_FAST_THREADS 128
#endif
#ifndef MPF_FAST_MINB
#define MPF_FAST_MINB 2
#endif
// Jacobian gathers unrolled per loop trip (1: one at a time)
#ifndef MPF_JAC_UNROLL
#define MPF_JAC_UNROLL 1
#endif
constexpr int kJacUnroll = MPF_JAC_UNROLL;
// TSC record gathers: 1 = a loop over the three x-slabs, 0 = fully unrolled
#ifndef MPF_TSC_SLAB
#define MPF_TSC_SLAB 0
#endif
constexpr int kFastThreads = MPF_FAST_THREADS;

// Utility::interpolate with the uniform index table (same bracketing interval
// as the reference's upper_bound; slope precomputed per interval).
__device__ __forceinline__ double interp_fast(const DevCosmo& C, double x0, const double* __restrict__ y,
                                              const double* __restrict__ slope)
{
    int i;
    if (x0 < C.t0) {
        i = 0;
    } else {
        const double kk = (x0 - C.t0) * C.lut_scale;
        const int k = (kk < (double)C.nlut) ? (int)kk : C.nlut;
        i = __ldg(C.lut + k);
        while (i < C.n && !(x0 < __ldg(C.t + i))) ++i;
    }
    const int n = C.n;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n <= 1) return (n > 0) ? __ldg(y) : 0.0;
    return __ldg(y + i - 1) + __ldg(slope + i - 1) * (x0 - __ldg(C.t + i - 1));
}

// Upper-bound position of x0 in the cosmology table (the bracket
// Utility::interpolate uses), from the uniform index table.
__device__ __forceinline__ int bracket_lut(const DevCosmo& C, double x0)
{
    if (x0 < C.t0) return 0;
    const double kk = (x0 - C.t0) * C.lut_scale;
    const int k = (kk < (double)C.nlut) ? (int)kk : C.nlut;
    int i = __ldg(C.lut + k);
    while (i < C.n && !(x0 < __ldg(C.t + i))) ++i;
    return i;
}

// Utility::interpolate with the bracket carried from the previous call: a
// ray's conformal time moves by much less than a table interval between two
// calls, so `first` (the upper bound of x0) is re-checked, not searched.
__device__ __forceinline__ double interp_cached(const DevCosmo& C, double x0, const double* __restrict__ y,
                                                const double* __restrict__ slope, int& first)
{
    const int n = C.n;
    while (first < n && !(x0 < __ldg(C.t + first))) ++first;
    while (first > 0 && x0 < __ldg(C.t + first - 1)) --first;
    int i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n <= 1) return (n > 0) ? __ldg(y) : 0.0;
    return __ldg(y + i - 1) + __ldg(slope + i - 1) * (x0 - __ldg(C.t + i - 1));
}

__device__ __forceinline__ void tsc_w3(float f, float* w)
{
    const float m = 0.5f - f, p = 0.5f + f;
    w[0] = 0.5f * m * m;
    w[1] = 0.75f - f * f;
    w[2] = 0.5f * p * p;
}

// integer coordinates at level L and the offset of the point from its cell
// centre in cell units (exact scaling by 2^L / EXTENT)
__device__ __forceinline__ void point_cell(int L, double x, double y, double z, uint32_t* c, float* fd)
{
    const double s = pow2(L - kLevelShift);   // 2^L / EXTENT, exact
    const double u[3] = {(x + 2.0) * s, (y + 2.0) * s, (z + 2.0) * s};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double f = floor(u[d]);
        c[d] = (f > 0.0) ? (uint32_t)(uint64_t)f : 0u;
        fd[d] = (float)(u[d] - f) - 0.5f;
    }
}

__device__ __forceinline__ int rec_flags(const DevTree& T, int cell) { return __ldg(&T.stencil[8 * (size_t)cell + 6].w); }
__device__ __forceinline__ int rec_entry(const DevTree& T, int cell, int j)
{
    return __ldg(reinterpret_cast<const int*>(T.stencil + 8 * (size_t)cell) + j);
}

// stats slots
enum { ST_RK_REC = 0, ST_RK_SLOW, ST_POST_REC, ST_POST_SLOW, ST_JAC_REC, ST_JAC_SLOW, ST_CELL_CHANGE, ST_STEPS, ST_N };

__device__ __forceinline__ void stat(unsigned long long* st, int k)
{
    if (st) atomicAdd(st + k, 1ull);
}

// Build-time diagnostics (-DMPF_DIAG=1): counts of the rare paths, read by
// the launcher when MPF_STATS is set.  [0] gather restarts at a coarser
// cell, [1] full walks from the top grid.
#if MPF_DIAG
__device__ unsigned long long g_diag[4];
#define MPF_DIAG_COUNT(k) atomicAdd(&g_diag[k], 1ull)
#else
#define MPF_DIAG_COUNT(k) ((void)0)
#endif

// Out-of-line slow paths (reference semantics with full walks), single copies
// so that the hot loop stays small in the instruction cache.
static __device__ __noinline__ Field7 tsc_slow(const DevTree& T, double x, double y, double z, int need_all)
{
    return tsc<false>(T, x, y, z, need_all != 0);
}
static __device__ __noinline__ Field7 cic_slow(const DevTree& T, double x, double y, double z, int need_all)
{
    return cic<false>(T, x, y, z, need_all != 0);
}
static __device__ __noinline__ Found locate_slow(const DevTree& T, double x, double y, double z) { return locate(T, x, y, z); }
// the 7 fields and the velocity, full walk (velocity-field octrees)
static __device__ __noinline__ Field7 vel_slow(const DevTree& T, int order, double x, double y, double z, float* v)
{
    return gather_vel<false>(T, order, x, y, z, v);
}

// A point given by its float64 coordinates.
struct PosAt {
    double x, y, z;
    __device__ __forceinline__ double px() const { return x; }
    __device__ __forceinline__ double py() const { return y; }
    __device__ __forceinline__ double pz() const { return z; }
};

// An RK stage point, b + c k: its float64 coordinates are formed only where a
// rare path (a full walk, a restart at a coarser cell) needs them; the common
// path works on the FP32 offset from the step's start cell.
struct PosStage {
    double bx, by, bz, dlL;
    float cfr, kx, ky, kz;   // converted to float64 on the rare paths only
    __device__ __forceinline__ double c() const { return (double)cfr * dlL; }
    __device__ __forceinline__ double px() const { return fma(c(), (double)kx, bx); }
    __device__ __forceinline__ double py() const { return fma(c(), (double)ky, by); }
    __device__ __forceinline__ double pz() const { return fma(c(), (double)kz, bz); }
};

// A located point: its deepest cell, that cell's level, integer coordinates
// and centre, and the point's offset from the centre in cell units.
struct Loc {
    int cell;
    int level;
    uint32_t c[3];
    double cen[3];
    float fd[3];
};

__device__ __forceinline__ float cells_per_unit(int L) { return __int_as_float((127 + L - kLevelShift) << 23); }

// full location by a walk from the top grid (float64 coordinates)
static __device__ __noinline__ Loc locate_full(const DevTree& T, double x, double y, double z)
{
    MPF_DIAG_COUNT(1);
    Loc r;
    const Found f = locate(T, x, y, z);
    r.cell = f.cell;
    r.level = f.level;
    if (f.cell >= 0) {
        point_cell(f.level, x, y, z, r.c, r.fd);
        for (int d = 0; d < 3; ++d) r.cen[d] = coord_center(f.level, r.c[d]);
    }
    return r;
}

// A point in the neighbour e (record entry (ox, oy, oz) of the located cell
// h) when e is not a leaf of h's level: a refined cell of h's level (the
// point's deepest cell is found by following e's children along the point's
// octants) or a coarser leaf (the point lies in it).  fx, fy, fz: the point's
// offset from the neighbour's centre in units of h's cells.  The tree is
// navigated through the node array and the offsets carried in FP32, instead
// of a float64 walk from the top grid; r.cell = -2 when neither case applies
// (a wrapped key, a partly refined node) and the caller walks.
static __device__ __noinline__ Loc neighbour_other(const DevTree& T, const Loc& h, int e, int fl, int ox, int oy, int oz,
                                            float fx, float fy, float fz)
{
    Loc r;
    r.cell = -2;
    const int L = h.level;
    const int le = fl & 255;
    const uint32_t lim = (uint32_t)((1ull << L) - 1ull);
    const uint32_t nc[3] = {h.c[0] + (uint32_t)ox, h.c[1] + (uint32_t)oy, h.c[2] + (uint32_t)oz};
    if (nc[0] > lim || nc[1] > lim || nc[2] > lim) return r;
    if (le == L && (fl & 256)) {
        const double w = cell_extent(L);
        double cen[3] = {h.cen[0] + (ox > 0 ? w : (ox < 0 ? -w : 0.0)), h.cen[1] + (oy > 0 ? w : (oy < 0 ? -w : 0.0)),
                         h.cen[2] + (oz > 0 ? w : (oz < 0 ? -w : 0.0))};
        uint32_t c[3] = {nc[0], nc[1], nc[2]};
        float f[3] = {fx, fy, fz};
        int cell = e, lev = L;
        int nd = __ldg(&T.stencil[8 * (size_t)e + 7].y);
        for (int guard = 0; guard < kMaxLevel; ++guard) {
            const int2 node = __ldg(T.node + nd);
            if (node.x < 0) break;   // e's descendant containing the point is a leaf
            const int b[3] = {f[0] >= 0.f ? 1 : 0, f[1] >= 0.f ? 1 : 0, f[2] >= 0.f ? 1 : 0};
            const int nd2 = node.x + (b[0] | (b[1] << 1) | (b[2] << 2));
            const int2 child = __ldg(T.node + nd2);
            if (child.y < 0) return r;
            const double q = pow2(kLevelShift - lev - 2);   // half the child's size
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                cen[d] += b[d] ? q : -q;
                c[d] = 2u * c[d] + (uint32_t)b[d];
                f[d] = 2.f * f[d] + 0.5f - (float)b[d];
            }
            cell = child.y;
            nd = nd2;
            ++lev;
        }
        r.cell = cell;
        r.level = lev;
#pragma unroll
        for (int d = 0; d < 3; ++d) { r.c[d] = c[d]; r.cen[d] = cen[d]; r.fd[d] = f[d]; }
        return r;
    }
    if (le < L && !(fl & 256)) {
        const int k = L - le;
        const float sk = __int_as_float((127 - k) << 23);   // 2^-k
        const float fn[3] = {fx, fy, fz};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            r.c[d] = nc[d] >> k;
            const uint32_t low = nc[d] - (r.c[d] << k);
            r.fd[d] = ((float)low + 0.5f + fn[d]) * sk - 0.5f;
            r.cen[d] = coord_center(le, r.c[d]);
        }
        r.cell = e;
        r.level = le;
        return r;
    }
    return r;
}

// Ancestor of a located cell at the coarser level lc, through the parents
// stored in the records; c and fd follow (fd' = (fd + bit - 1/2) / 2 per
// level).  -1 when a parent is missing.
__device__ __forceinline__ int ancestor_up(const DevTree& T, int cell, int L, int lc, uint32_t* c, float* fd)
{
    for (int guard = 0; guard < kMaxLevel && L > lc; ++guard) {
        const int p = __ldg(&T.stencil[8 * (size_t)cell + 7].z);
        if (p < 0) return -1;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            fd[d] = (fd[d] + (float)(c[d] & 1u) - 0.5f) * 0.5f;
            c[d] >>= 1;
        }
        cell = p;
        --L;
    }
    return (L == lc) ? cell : -1;
}

// Deepest cell of point (x, y, z) given a nearby located cell `h`: the offset
// from h's centre is formed in float64 (one subtraction per axis) and the rest
// in FP32; the cell is h or one of its 26 neighbours read from h's record when
// that neighbour is a leaf of h's level; otherwise a full walk.
template <class P>
__device__ __forceinline__ Loc locate_rel(const DevTree& T, const Loc& h, float rx, float ry, float rz, const P& pos)
{
    if (h.cell >= 0) {
        const int ox = (int)floorf(rx + 0.5f), oy = (int)floorf(ry + 0.5f), oz = (int)floorf(rz + 0.5f);
        if (ox == 0 && oy == 0 && oz == 0) {
            Loc r = h;
            r.fd[0] = rx; r.fd[1] = ry; r.fd[2] = rz;
            return r;
        }
        if (abs(ox) <= 1 && abs(oy) <= 1 && abs(oz) <= 1) {
            const int e = rec_entry(T, h.cell, (ox + 1) * 9 + (oy + 1) * 3 + (oz + 1));
            if (e >= 0) {
                const int fl = rec_flags(T, e);
                if (!(fl & 256) && (fl & 255) == h.level) {
                    Loc r;
                    r.cell = e;
                    r.level = h.level;
                    const double w = cell_extent(h.level);
                    r.c[0] = h.c[0] + ox; r.c[1] = h.c[1] + oy; r.c[2] = h.c[2] + oz;
                    // +-w or 0 per axis (selects, no int-to-double conversion)
                    r.cen[0] = h.cen[0] + (ox > 0 ? w : (ox < 0 ? -w : 0.0));
                    r.cen[1] = h.cen[1] + (oy > 0 ? w : (oy < 0 ? -w : 0.0));
                    r.cen[2] = h.cen[2] + (oz > 0 ? w : (oz < 0 ? -w : 0.0));
                    r.fd[0] = rx - (float)ox; r.fd[1] = ry - (float)oy; r.fd[2] = rz - (float)oz;
                    return r;
                }
                const Loc r = neighbour_other(T, h, e, fl, ox, oy, oz, rx - (float)ox, ry - (float)oy, rz - (float)oz);
                if (r.cell != -2) return r;
            }
        }
    }
    return locate_full(T, pos.px(), pos.py(), pos.pz());
}

// Deepest cell of a point given by float64 coordinates near a located cell:
// the offset from the cell's centre is formed in float64 (one subtraction per
// axis) and rounded to FP32 cell units.
__device__ __forceinline__ Loc locate_near(const DevTree& T, const Loc& h, double x, double y, double z)
{
    float rx = 0.f, ry = 0.f, rz = 0.f;
    if (h.cell >= 0) {
        const float sc = cells_per_unit(h.level);
        rx = (float)(x - h.cen[0]) * sc; ry = (float)(y - h.cen[1]) * sc; rz = (float)(z - h.cen[2]) * sc;
    }
    return locate_rel(T, h, rx, ry, rz, PosAt{x, y, z});
}

// The point one cell away from a located point along an axis: same in-cell
// offset, neighbouring cell from the record (the six Jacobian points).
__device__ __forceinline__ Loc step_cell(const DevTree& T, const Loc& h, int axis, int sgn, double x, double y, double z)
{
    const int ox = axis == 0 ? sgn : 0, oy = axis == 1 ? sgn : 0, oz = axis == 2 ? sgn : 0;
    const int e = rec_entry(T, h.cell, (ox + 1) * 9 + (oy + 1) * 3 + (oz + 1));
    if (e >= 0) {
        const int fl = rec_flags(T, e);
        if (!(fl & 256) && (fl & 255) == h.level) {
            Loc r = h;
            r.cell = e;
            const double sw = (sgn > 0) ? cell_extent(h.level) : -cell_extent(h.level);
            r.c[0] += ox; r.c[1] += oy; r.c[2] += oz;
            const double moved = ((axis == 0) ? h.cen[0] : (axis == 1) ? h.cen[1] : h.cen[2]) + sw;
            if (axis == 0) r.cen[0] = moved;
            else if (axis == 1) r.cen[1] = moved;
            else r.cen[2] = moved;
            return r;
        }
        const Loc r = neighbour_other(T, h, e, fl, ox, oy, oz, h.fd[0], h.fd[1], h.fd[2]);
        if (r.cell != -2) return r;
    }
    return locate_full(T, x, y, z);
}

// TSC at a point whose deepest cell is `cell` (simplehyperoctree.h:1479-1541
// through the stencil records).  Returns false when a restart centre is not
// itself a cell (left to the slow path).
// VEL: also the velocity slots into vv[3] (with need_all).
template <bool VEL, class P>
__device__ __forceinline__ bool tsc_rec(const DevTree& T, const Loc& d, const P& pos, bool need_all, Field7& res, float* vv)
{
    int cell = d.cell, L = d.level;
    float fd[3] = {d.fd[0], d.fd[1], d.fd[2]};
    uint32_t c[3] = {d.c[0], d.c[1], d.c[2]};
    for (int guard = 0; guard <= kMaxLevel; ++guard) {
        const int4* rp = T.stencil + 8 * (size_t)cell;
        const int4 r7 = __ldg(rp + 7);
        const unsigned exact = (unsigned)r7.x;
        if (exact == kFullMask) {
            float wx[3], wy[3], wz[3];
            tsc_w3(fd[0], wx);
            tsc_w3(fd[1], wy);
            tsc_w3(fd[2], wz);
            float gx = 0.f, gy = 0.f, gz = 0.f, gt = 0.f, rho = 0.f, phi = 0.f, a = 0.f;
            float ux = 0.f, uy = 0.f, uz = 0.f;
#if MPF_TSC_SLAB
            // one x-slab of 9 cells per loop trip: a third of the code of the
            // fully unrolled loop (the kernel is instruction-fetch bound)
            const int* re = reinterpret_cast<const int*>(rp);
#pragma unroll 1
            for (int ix = 0; ix < 3; ++ix) {
                const float wxi = (ix == 0) ? wx[0] : ((ix == 1) ? wx[1] : wx[2]);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    const int e = __ldg(re + 9 * ix + k);
                    const float wt = wxi * wy[k / 3] * wz[k % 3];
                    const float4 g = __ldg(T.grad + e);
                    gx = fmaf(g.x, wt, gx); gy = fmaf(g.y, wt, gy); gz = fmaf(g.z, wt, gz); gt = fmaf(g.w, wt, gt);
                    if (need_all) {
                        const float4 s = __ldg(T.scal + e);
                        rho = fmaf(s.x, wt, rho); phi = fmaf(s.y, wt, phi); a = fmaf(s.z, wt, a);
                        if (VEL) {
                            const float4 u = __ldg(T.vel + e);
                            ux = fmaf(u.x, wt, ux); uy = fmaf(u.y, wt, uy); uz = fmaf(u.z, wt, uz);
                        }
                    }
                }
            }
#else
            int e[28];
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                const int4 v = __ldg(rp + q);
                e[4 * q] = v.x; e[4 * q + 1] = v.y; e[4 * q + 2] = v.z; e[4 * q + 3] = v.w;
            }
#pragma unroll
            for (int j = 0; j < 27; ++j) {
                // wy * wz is shared by the three x-slabs: 9 products, then one per cell
                const float wt = wx[j / 9] * (wy[(j / 3) % 3] * wz[j % 3]);
                const float4 g = __ldg(T.grad + e[j]);
                gx = fmaf(g.x, wt, gx); gy = fmaf(g.y, wt, gy); gz = fmaf(g.z, wt, gz); gt = fmaf(g.w, wt, gt);
                if (need_all) {
                    const float4 s = __ldg(T.scal + e[j]);
                    rho = fmaf(s.x, wt, rho); phi = fmaf(s.y, wt, phi); a = fmaf(s.z, wt, a);
                    if (VEL) {
                        const float4 u = __ldg(T.vel + e[j]);
                        ux = fmaf(u.x, wt, ux); uy = fmaf(u.y, wt, uy); uz = fmaf(u.z, wt, uz);
                    }
                }
            }
#endif
            res = Field7{rho, phi, gx, gy, gz, a, gt};
            if (VEL) { vv[0] = ux; vv[1] = uy; vv[2] = uz; }
            return true;
        }
        // first entry (x-major) not at this level: missing -> empty, coarser -> restart there
        const int j = __ffs(~exact & kFullMask) - 1;
        const int e = __ldg(reinterpret_cast<const int*>(rp) + j);
        if (e < 0) {
            clear(res);
            if (VEL) vv[0] = vv[1] = vv[2] = 0.f;
            return true;
        }
        const int lc = rec_flags(T, e) & 255;
        MPF_DIAG_COUNT(0);
        // the restart cell is the point's ancestor at level lc
        const int up = ancestor_up(T, cell, L, lc, c, fd);
        if (up >= 0) {
            cell = up;
            L = lc;
            continue;
        }
        const double x = pos.px(), y = pos.py(), z = pos.pz();
        const Found f = find_cell(T, lc, axis_coord(lc, x), axis_coord(lc, y), axis_coord(lc, z));
        if (f.cell < 0 || f.level != lc) return false;
        cell = f.cell;
        L = lc;
        point_cell(L, x, y, z, c, fd);
    }
    return false;
}

// CIC at a point whose deepest cell is `cell` (simplehyperoctree.h:1410-1469).
template <bool VEL, class P>
__device__ __forceinline__ bool cic_rec(const DevTree& T, const Loc& d, const P& pos, bool need_all, Field7& res, float* vv)
{
    int cell = d.cell, L = d.level;
    float fd[3] = {d.fd[0], d.fd[1], d.fd[2]};
    uint32_t c[3] = {d.c[0], d.c[1], d.c[2]};
    for (int guard = 0; guard <= kMaxLevel; ++guard) {
        const int sx = (fd[0] >= 0.f) ? 1 : -1, sy = (fd[1] >= 0.f) ? 1 : -1, sz = (fd[2] >= 0.f) ? 1 : -1;
        const float ax = fabsf(fd[0]), ay = fabsf(fd[1]), az = fabsf(fd[2]);
        int lvl = L;
        bool missing = false;
        float gx = 0.f, gy = 0.f, gz = 0.f, gt = 0.f, rho = 0.f, phi = 0.f, a = 0.f;
        float ux = 0.f, uy = 0.f, uz = 0.f;
        for (int v = 0; v < 8; ++v) {
            const int ox = (v & 1) ? ((sx > 0) ? 1 : 0) : ((sx > 0) ? 0 : -1);
            const int oy = (v & 2) ? ((sy > 0) ? 1 : 0) : ((sy > 0) ? 0 : -1);
            const int oz = (v & 4) ? ((sz > 0) ? 1 : 0) : ((sz > 0) ? 0 : -1);
            const int e = rec_entry(T, cell, (ox + 1) * 9 + (oy + 1) * 3 + (oz + 1));
            if (e < 0) { missing = true; break; }
            const int le = rec_flags(T, e) & 255;
            lvl = min(lvl, le);
            // the neighbour cell gets |fd|, the centre cell 1 - |fd| (per axis)
            const float wt = (ox ? ax : 1.f - ax) * (oy ? ay : 1.f - ay) * (oz ? az : 1.f - az);
            const float4 g = __ldg(T.grad + e);
            gx = fmaf(g.x, wt, gx); gy = fmaf(g.y, wt, gy); gz = fmaf(g.z, wt, gz); gt = fmaf(g.w, wt, gt);
            if (need_all) {
                const float4 s = __ldg(T.scal + e);
                rho = fmaf(s.x, wt, rho); phi = fmaf(s.y, wt, phi); a = fmaf(s.z, wt, a);
                if (VEL) {
                    const float4 u = __ldg(T.vel + e);
                    ux = fmaf(u.x, wt, ux); uy = fmaf(u.y, wt, uy); uz = fmaf(u.z, wt, uz);
                }
            }
        }
        if (lvl == L) {
            if (missing) clear(res);
            else res = Field7{rho, phi, gx, gy, gz, a, gt};
            if (VEL) {
                vv[0] = missing ? 0.f : ux; vv[1] = missing ? 0.f : uy; vv[2] = missing ? 0.f : uz;
            }
            return true;
        }
        MPF_DIAG_COUNT(0);
        const int up = ancestor_up(T, cell, L, lvl, c, fd);
        if (up >= 0) {
            cell = up;
            L = lvl;
            continue;
        }
        const double x = pos.px(), y = pos.py(), z = pos.pz();
        const Found f = find_cell(T, lvl, axis_coord(lvl, x), axis_coord(lvl, y), axis_coord(lvl, z));
        if (f.cell < 0 || f.level != lvl) return false;
        cell = f.cell;
        L = lvl;
        point_cell(L, x, y, z, c, fd);
    }
    return false;
}

// maybe_origin: the point can be the exact origin (first step of a ray),
// where the reference's TSC falls back to CIC (simplehyperoctree.h:1570-1571)
// VEL (with need_all): the velocity slots into vv[3] as well.
template <int ORDER, bool VEL = false, class P>
__device__ __forceinline__ Field7 gather_at(const DevTree& T, const Loc& d, const P& pos, bool need_all,
                                            unsigned long long* st, int slot, bool maybe_origin, float* vv = nullptr)
{
    constexpr int order = ORDER;
    Field7 r;
    if (d.cell < 0) {
        clear(r);
        if (VEL) vv[0] = vv[1] = vv[2] = 0.f;
        stat(st, slot);
        return r;
    }
    if (!(maybe_origin && pos.px() == 0.0 && pos.py() == 0.0 && pos.pz() == 0.0)) {
        const bool ok = (order == 1) ? cic_rec<VEL>(T, d, pos, need_all, r, vv) : tsc_rec<VEL>(T, d, pos, need_all, r, vv);
        if (ok) {
            stat(st, slot);
            return r;
        }
    }
    stat(st, slot + 1);
    if (VEL && need_all) return vel_slow(T, order, pos.px(), pos.py(), pos.pz(), vv);
    return (order == 1) ? cic_slow(T, pos.px(), pos.py(), pos.pz(), need_all)
                        : tsc_slow(T, pos.px(), pos.py(), pos.pz(), need_all);
}

struct FastRec {
    double a, t, x, y, z, k0, k1, k2, k3;
    double phi, red, chi, lambda, s, isw, iswold;
    double dop;   // velocity-field octrees: the point's Doppler term v.k / (c k0)
    float rho, dx, dy, dz, dt, ah;   // dt: the photon's (forward) dphidt
    int level;
};

// 1/a: FP32 seed refined by two Newton steps (full float64 accuracy)
__device__ __forceinline__ double recip(double a)
{
    double r = (double)(1.0f / (float)a);
    r = fma(r, fma(-a, r, 1.0), r);
    r = fma(r, fma(-a, r, 1.0), r);
    return r;
}


// geodesic RHS (integrator.h:409-445) from the field at the point.
// in = (a, t, x, y, z, k0, k1, k2, k3).  The FP64 pipe of this GPU retires 2
// operations per cycle per SM (1/64 of FP32), so the RHS keeps in FP64 only
// what the trajectory's accuracy needs:
//  * dphi/dlambda and the terms built from it are FP32: they only enter as
//    (2/c^2) dphi/dlambda, a rate that multiplies k (its error changes |k| by
//    a relative 1e-7 of that term's increment, not the direction);
//  * the lensing source 2 dphi/dx^i k0^2 is an FP32 product (the field is FP32);
//  * the Hubble drag and the k^i multiplications stay FP64, so the direction
//    of k and the positions keep float64 accuracy;
//  * dx/dlambda is returned as k itself: the caller folds 1/scale into the
//    RK coefficient (one multiplication per stage instead of three).
// inv_a = 1 / in[0]; tb = the cosmology bracket carried along the ray.
// kf: k^1..k^3 rounded to FP32 (the next stage's point offset in cell units).
__device__ __forceinline__ void rhs_math(const DevCosmo& C, const Field7& g, const double* in, double inv_a, int& tb,
                                         double* out, float* kf)
{
    const double c2 = kC * kC;
    const float k0f = (float)in[5], k1f = (float)in[6], k2f = (float)in[7], k3f = (float)in[8];
    kf[0] = k1f; kf[1] = k2f; kf[2] = k3f;
    const float dphidl = g.dt * k0f + (g.dx * k1f + g.dy * k2f + g.dz * k3f);
    const double dadt = interp_cached(C, in[1], C.dadt, C.slope_dadt, tb);
    out[0] = in[5] * dadt;
    out[1] = in[5];
    out[2] = in[6];
    out[3] = in[7];
    out[4] = in[8];
    const double hub = 2.0 * out[0] * inv_a;
    const float two_c2 = (float)(2.0 / c2);
    const float k02 = 2.0f * k0f * k0f;
    out[5] = -(hub * in[5]) - (double)((two_c2 * k0f) * (dphidl - g.dt * k0f));
    const double coef = (double)(two_c2 * dphidl) - hub;
    out[6] = fma(coef, in[6], -(double)(g.dx * k02));
    out[7] = fma(coef, in[7], -(double)(g.dy * k02));
    out[8] = fma(coef, in[8], -(double)(g.dz * k02));
}

// The photon record (Photon<double,3> fields) of a fast-mode trajectory point;
// data_dt: the field's dphidt there, dphi_over_dl: the laplacian column
// ((phi - previous phi) / dl), k: the point's index.
__device__ __forceinline__ Rec fast_record(const FastRec& b, float data_dt, double dphi_over_dl, long long k)
{
    const double c2 = kC * kC;
    Rec r;
    r.a = b.a; r.t = b.t; r.x = b.x; r.y = b.y; r.z = b.z; r.k0 = b.k0; r.k1 = b.k1; r.k2 = b.k2; r.k3 = b.k3;
    r.level = b.level; r.ah = b.ah; r.rho = b.rho; r.phi = b.phi;
    r.dx = b.dx; r.dy = b.dy; r.dz = b.dz; r.dt = b.dt;
    r.dphidl = (k > 0) ? ((double)data_dt * b.k0 + ((double)b.dx * b.k1 + (double)b.dy * b.k2 + (double)b.dz * b.k3)) : 0.0;
    r.lap = (k > 0) ? dphi_over_dl : 0.0;
    const double kk = b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3;
    r.ds2 = (b.a * b.a) * (-(c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0) + ((1.0 - 2.0 * (b.phi / c2)) * kk));
    r.err = 1.0 - ((1.0 - 2.0 * (b.phi / c2)) * kk) / (c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0);
    r.red = b.red; r.isw = b.isw; r.iswold = b.iswold; r.chi = b.chi; r.lambda = b.lambda; r.s = b.s;
    r.index = (double)k;
    return r;
}

// Jacobian terms (d1d1, d1d2, d2d2 of lensing.h:430-447) at a trajectory
// point located at `here`: six TSC gathers at +-1 cell.
__device__ __forceinline__ void jac_fast(const DevTree& T, const Loc& here, double x, double y, double z, float* out3,
                                         unsigned long long* st)
{
    // dl = 2^-(level - 1 - log2 EXTENT) (lensing.h:430); h = dl / 2 = one cell of the point's level
    const double h = pow2(kLevelShift - here.level);
    float g[6][3];
#pragma unroll kJacUnroll
    for (int a = 0; a < 6; ++a) {
        const int ax = a >> 1;
        const int sgn = (a & 1) ? 1 : -1;
        const double moved = ((ax == 0) ? x : (ax == 1) ? y : z) + ((a & 1) ? h : -h);
        const double qx = (ax == 0) ? moved : x, qy = (ax == 1) ? moved : y, qz = (ax == 2) ? moved : z;
        const Loc d = step_cell(T, here, ax, sgn, qx, qy, qz);
        const Field7 f = gather_at<2>(T, d, PosAt{qx, qy, qz}, false, st, ST_JAC_REC, false);
        g[a][0] = f.dx; g[a][1] = f.dy; g[a][2] = f.dz;
    }
    const float idl = __int_as_float((127 + here.level - kLevelShift - 1) << 23);   // 1 / dl, exact
    const float dxx = (g[1][0] - g[0][0]) * idl, dxy = (g[3][0] - g[2][0]) * idl, dxz = (g[5][0] - g[4][0]) * idl;
    const float dyy = (g[3][1] - g[2][1]) * idl, dyz = (g[5][1] - g[4][1]) * idl, dzz = (g[5][2] - g[4][2]) * idl;
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    const float rho = sqrtf(fx * fx + fy * fy);
    const float r = sqrtf(fx * fx + fy * fy + fz * fz);
    const float cp = (rho > 0.f) ? fx / rho : 1.f, sp = (rho > 0.f) ? fy / rho : 0.f;
    const float ct = fz / r, snt = rho / r;
    const float s2p = 2.f * sp * cp, s2t = 2.f * snt * ct;
    out3[0] = sp * sp * dxx + cp * cp * dyy - s2p * dxy;
    out3[1] = ct * cp * sp * (dyy - dxx) + (cp * cp - sp * sp) * ct * dxy + sp * snt * dxz - cp * snt * dyz;
    out3[2] = cp * cp * ct * ct * dxx + sp * sp * ct * ct * dyy + snt * snt * dzz + s2p * ct * ct * dxy - sp * s2t * dyz -
              cp * s2t * dxz;
}

// Per-thread Jacobian running sums kept in shared memory (touched once per
// step, so they need not occupy registers through the gathers): the FP64
// sums S (6), and the last point's contribution c_k (6) and the one before it
// c_km1 (6), FP32 products of the point's FP32 Hessian terms; strided by the
// block size.
struct JacSums {
    double* sums;   // this thread's slot 0 of S
    float* terms;   // this thread's slot 0 of c_k, c_km1
    __device__ __forceinline__ double& S(int q) const { return sums[q * kFastThreads]; }
    __device__ __forceinline__ float& ck(int q) const { return terms[q * kFastThreads]; }
    __device__ __forceinline__ float& ckm1(int q) const { return terms[(6 + q) * kFastThreads]; }
};

// SRC: source mode (one surface at the ray's own radius); WIDE: per-ray
// surfaces and wide surface records (bundle rays).  The plain instantiation,
// the map and benchmark path, carries neither.  VEL: a velocity-field octree
// (the reference's -DVELOCITYFIELD build): the post-step gathers also read
// the velocity slots, an all-zero record with a velocity is not empty, and
// the redshift takes the ISW, Doppler and observer terms
// (integrator.h:707-708, 765-767); plain instantiations only.
template <int ORDER, bool SRC, bool WIDE, bool BORN = false, bool VEL = false>
__device__ void propagate_fast(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* L, long long i,
                               const PropOut& O, JacSums J)
{
    const double c2 = kC * kC;
    const double mn = -(double)kExtent / 2.0, mx = (double)kExtent / 2.0;
    const double scale = P.length;
    const double inv_scale = 1.0 / scale;
    const int np = SRC ? 1 : P.nplanes;
    const int skind = SRC ? (int)STOP_R : P.stop_kind;
    const double* rpl = (WIDE && P.ray_planes) ? P.ray_planes + i * np : P.planes;   // this ray's surfaces
    const double stop_ref = SRC ? P.ray_stop[i] : ((WIDE && P.ray_planes) ? rpl[np - 1] : P.stop_ref);
    const int rec_fields = SRC ? kSourceFields : (WIDE ? kWideFields : kPlaneFields);
    unsigned long long* const st = O.stats;
    // Born ray (Order = -1 on the octree itself: hmaps.h:706-712,
    // catalogues.h:670-673), an instantiation of its own: the homogeneous
    // field in the stages and after each step, the octree's levels for the
    // step length, its field for the Jacobian
    constexpr bool born = BORN;
    Field7 hom;
    clear(hom);
    hom.a = 1.f;
    FastRec b;
    if (SRC || (WIDE && P.direct)) {
        // (phi, theta) launch form or a bundle photon: the direction is given
        b.a = 1.0; b.t = 0.0; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = 1.0;
        b.k1 = L[3]; b.k2 = L[4]; b.k3 = L[5];
    } else {
        const double norm = sqrt((L[3] - L[0]) * (L[3] - L[0]) + (L[4] - L[1]) * (L[4] - L[1]) + (L[5] - L[2]) * (L[5] - L[2]));
        b.a = 1.0; b.t = 0.0; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = 1.0;
        b.k1 = (L[3] - L[0]) / norm; b.k2 = (L[4] - L[1]) / norm; b.k3 = (L[5] - L[2]) / norm;
    }
    Loc here = locate_full(T, b.x, b.y, b.z);
    float vv[3] = {0.f, 0.f, 0.f};   // VEL: the velocity of the last post-step gather
    Field7 data = born ? hom : gather_at<ORDER, VEL>(T, here, PosAt{b.x, b.y, b.z}, true, st, ST_POST_REC, true, vv);
    {
        const double ph = (double)data.phi / c2;
        const double norm = sqrt((c2 * (1.0 + 2.0 * ph) * b.k0 * b.k0) / ((1.0 - 2.0 * ph) * (b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3)));
        b.k1 *= norm; b.k2 *= norm; b.k3 *= norm;
    }
    const double v0n = VEL ? (P.vobs[0] * b.k1 + P.vobs[1] * b.k2 + P.vobs[2] * b.k3) / (kC * b.k0) : 0.0;
    b.dop = 0.0;
    // data != empty (integrator.h:715): with VEL the velocity slots count too
    auto empty = [&]() -> bool { return is_empty(data) && (!VEL || (vv[0] == 0.f && vv[1] == 0.f && vv[2] == 0.f)); };
    b.a = interp_fast(C, b.t, C.a, C.slope_a);
    b.level = (here.cell >= 0) ? here.level : 0;
    b.ah = 0.f;
    b.rho = data.rho; b.phi = data.phi; b.dx = data.dx; b.dy = data.dy; b.dz = data.dz; b.dt = data.dt;
    b.red = 0.0; b.isw = 0.0; b.chi = 0.0; b.iswold = 0.0; b.lambda = 0.0; b.s = 0.0;
    const double ratio_k = (scale / kC) / P.nsteps;
    double ratio = b.a * b.a * ratio_k;
    double dl = (here.cell >= 0 ? cell_extent(here.level) : 0.0) * ratio;
    const double a0 = b.a;
    int tb = bracket_lut(C, b.t);       // cosmology-table bracket of the ray's conformal time
    const double phi0c2 = b.phi / c2;
    float last_data_dt = data.dt;
    float last_dphi = 0.f;
    double last_dl = 1.0;

    // every trajectory point (bundle rays), wide instantiation only
    double* const traj = (WIDE && O.traj) ? O.traj + i * O.traj_cap * kPhotonFields : nullptr;
    if (WIDE && traj && O.traj_cap > 0) write_rec(traj, fast_record(b, 0.f, 0.0, 0));
    int next_plane = 0;
    long long cross_k[kMaxPlanes];
    for (int j = 0; j < np; ++j) cross_k[j] = -1;
    double* prow = O.plane_rec ? O.plane_rec + (long long)i * np * rec_fields : nullptr;
    if (SRC && prow) {
        prow[24] = b.a; prow[25] = b.phi; prow[26] = b.k1; prow[27] = b.k2; prow[28] = b.k3;
        prow[29] = prow[30] = prow[31] = 0.0;
    }
    // this ray's plane normals (stop criterion "plane" with per-ray surfaces; wide instantiation)
    const double* rki = (WIDE && P.ray_ki) ? P.ray_ki + i * np * 3 : nullptr;
    auto start_q = [&](int jn) -> double {
        if (rki && skind == STOP_PLANE) return b.x * rki[3 * jn] + b.y * rki[3 * jn + 1] + b.z * rki[3 * jn + 2];
        return (skind == STOP_R) ? b.chi : (skind == STOP_LAMBDA) ? b.lambda : (skind == STOP_T) ? b.t
             : (skind == STOP_S) ? b.s : b.red;
    };
    while (next_plane < np && ((skind == STOP_A) ? (b.a < (SRC ? stop_ref : rpl[next_plane]))
                                                  : (start_q(next_plane) > (SRC ? stop_ref : rpl[next_plane])))) {
        cross_k[next_plane] = 0;
        ++next_plane;
    }
    double rmax = 0.0;
    bool have_rmax = false;
    for (int q = 0; q < 6; ++q) { J.S(q) = 0.0; J.ck(q) = 0.f; J.ckm1(q) = 0.f; }
    double chim1 = 0.0, chim2 = 0.0;
    long long k = 0;
    unsigned status = 0;
    double isw = 0.0, iswold = 0.0, lambda = 0.0, sacc = 0.0;
    // A point's redshift (integrator.h:769) is formed only where it is read:
    // surface records, the end of the ray, trajectory records.  The stop and
    // crossing tests compare a0 (1 + phi0/c^2 - phi/c^2) with (1 + z) a
    // instead, which needs no division.  The starting point's redshift is 0.
    const double opc = 1.0 + phi0c2;
    const double inv_c2 = 1.0 / c2;
    // VEL: a0 / a (1 + phi0/c^2 - phi/c^2 + isw + v.k / (c k0) - v0n) - 1
    auto zbracket = [&](const FastRec& r) -> double {
        if (VEL) return opc - r.phi * inv_c2 + r.isw + r.dop - v0n;
        return opc - r.phi * inv_c2;
    };
    auto red_of = [&](const FastRec& r) -> double { return a0 * recip(r.a) * zbracket(r) - 1.0; };
    auto red_above = [&](const FastRec& r, double zref) -> bool { return a0 * zbracket(r) > (1.0 + zref) * r.a; };
    bool b_red_ok = true;     // b.red holds b's redshift
    const float two_c2 = (float)(2.0 / c2);
    const float inv_c2f = (float)(1.0 / c2);
    FastRec p;
    while (!empty()) {
        if (k >= P.max_steps) { status |= 1u; break; }
        // ---- RK4 step (integrator.h:718-734).  The state stays FP64 and is
        // accumulated in FP64; the four stages are evaluated in FP32 as
        // increments from the step's start b (c = 0, 1/2, 1/2, 1; weights
        // w = 1, 2, 2, 1):
        //   k_s = k_b + q_s,  q_s = c_s dl k'_{s-1},
        //   k^i' = coef k^i - 2 dphi/dx^i k0^2,   k0' = coef0 k0,
        //   coef = (2/c^2) dphi/dlambda - h,  coef0 = -h - (2/c^2) grad(phi).k,
        // with h = 2 (a'/a) k0 the Hubble drag (integrator.h:437-441).  The
        // drag sets |k| and the redshift, so it is formed once per step in FP64
        // at b, h_b, and each stage contributes its relative change
        // h_s = h_b (1 + eps_s) (eps ~ dl/L, FP32).  Then
        //   k^i_new = k^i_b + dl/6 (k^i_b sum w coef_s + sum w (coef_s q^i_s - 2 dphi/dx^i k0_s^2))
        //   x^i_new = x^i_b + dl/L k^i_b + dl/(6 L) sum w q^i_s
        //   t_new   = t_b + dl k0_b + dl/6 sum w q0_s
        //   a_new   = a_b + dl k0_b a'_b (1 + sum w ((1 + u_s)(1 + q0_s / k0_b) - 1) / 6)
        // with u_s the stage's relative change of a'.  The terms that set the
        // direction of k, |k| and the positions (k_b times the FP64 rates,
        // dl k_b) are FP64 products; the FP32 parts are corrections of
        // relative size dl/L (1e-4 to 1e-3 of the state).
        // da/dt at b (FP64, from the bracket carried along the ray) and the
        // distance to the bracket's upper node; the stages' da/dt follow the
        // table's linear pieces in FP32 from there.
        int ib;
        double adb;
        float tnext;
        {
            const int n = C.n;
            while (tb < n && !(b.t < __ldg(C.t + tb))) ++tb;
            while (tb > 0 && b.t < __ldg(C.t + tb - 1)) --tb;
            ib = tb + (n > 1) * ((tb <= 0) - (tb >= n));
            if (n > 1) {
                adb = __ldg(C.dadt + ib - 1) + __ldg(C.slope_dadt + ib - 1) * (b.t - __ldg(C.t + ib - 1));
                tnext = (ib < n - 1) ? (float)(__ldg(C.t + ib) - b.t) : __int_as_float(0x7f800000);
            } else {
                adb = (n > 0) ? __ldg(C.dadt) : 0.0;
                tnext = __int_as_float(0x7f800000);
            }
        }
        // da/dt(b.t + dt) - da/dt(b.t) along the table's pieces (dt >= 0; the
        // last piece extends past the table's end, as in Utility::interpolate)
        auto dadot = [&](float dt) -> float {
            if (C.n <= 1) return 0.f;
            float tn = tnext, rem = dt, r = 0.f;
            float sl = __ldg(&C.seg[ib - 1].x);
            int j = ib;
            for (int guard = 0; rem > tn && guard < 64; ++guard) {
                r = fmaf(sl, tn, r);
                rem -= tn;
                const float2 sj = __ldg(C.seg + j);
                sl = sj.x;
                tn = (j + 2 < C.n) ? sj.y : __int_as_float(0x7f800000);
                ++j;
            }
            return fmaf(sl, rem, r);
        };
        const double dlL = dl * inv_scale;
        const double hubb = 2.0 * adb * recip(b.a) * b.k0;
        const float dlf = (float)dl, dlLf = (float)dlL, hubbf = (float)hubb;
        const float kb0 = (float)b.k0, kb1 = (float)b.k1, kb2 = (float)b.k2, kb3 = (float)b.k3;
        const float abf = (float)b.a, adbf = (float)adb;
        const float inv_kb0 = 1.f / kb0, inv_adbf = (adbf != 0.f) ? 1.f / adbf : 0.f;
        const float cpu = cells_per_unit(here.level);
        // previous stage: its k' (d0..d3), a' (dA) and k (pk0..pk3)
        float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f, dA = 0.f;
        float pk0 = kb0, pk1 = kb1, pk2 = kb2, pk3 = kb3;
        // weighted sums over the stages: the gravitational parts of coef and
        // coef0 (Gd, Gk), the drag's relative changes (Se), the second-order
        // terms of k (E), the stage increments (S) and the a' terms (SA)
        float Gd = 0.f, Gk = 0.f, Se = 0.f, E0 = 0.f, E1 = 0.f, E2 = 0.f, E3 = 0.f;
        float S0 = 0.f, S1 = 0.f, S2 = 0.f, S3 = 0.f, SA = 0.f;
        float dtf;   // the step's conformal-time increment
#pragma unroll 1
        for (int sg = 0; sg < 4; ++sg) {
            const float cfr = (sg == 0) ? 0.f : ((sg < 3) ? 0.5f : 1.f);
            const float w = (sg == 0 || sg == 3) ? 1.f : 2.f;
            const float cdl = cfr * dlf;
            const float q0 = cdl * d0, q1 = cdl * d1, q2 = cdl * d2, q3 = cdl * d3;
            const float k0 = kb0 + q0, k1 = kb1 + q1, k2 = kb2 + q2, k3 = kb3 + q3;
            const float as = fmaf(cdl, dA, abf);
            const float dad = dadot(cdl * pk0);
            // stage 1 is at b, where the previous step's post-step gather read
            // the field (data); stages 2-4 are located from their FP32 offset
            // to b's cell, their float64 coordinates formed only on the rare
            // full-walk / restart paths
            Field7 g = data;
            if (sg > 0) {
                g = hom;
                if (!born) {
                    const float cc = cfr * dlLf * cpu;
                    const PosStage ps{b.x, b.y, b.z, dlL, cfr, pk1, pk2, pk3};
                    const Loc d = locate_rel(T, here, fmaf(cc, pk1, here.fd[0]), fmaf(cc, pk2, here.fd[1]),
                                             fmaf(cc, pk3, here.fd[2]), ps);
                    g = gather_at<ORDER>(T, d, ps, false, st, ST_RK_REC, false);
                }
            }
            const float gk = g.dx * k1 + (g.dy * k2 + g.dz * k3);
            const float dphidl = fmaf(g.dt, k0, gk);
            // the drag at the stage relative to b: a' (1 + u), a / (1 - v'), k0 (1 + wk)
            const float u = dad * inv_adbf, v = -(cdl * dA) / as, wk = q0 * inv_kb0;
            const float eps = u + v + wk + (u * v + u * wk + v * wk) + u * v * wk;
            const float hub = hubbf * (1.f + eps);
            const float coef = two_c2 * dphidl - hub;
            const float coef0 = -hub - two_c2 * gk;
            const float k02 = 2.f * k0 * k0;
            const float G1 = g.dx * k02, G2 = g.dy * k02, G3 = g.dz * k02;
            Gd = fmaf(w, two_c2 * dphidl, Gd);
            Gk = fmaf(w, two_c2 * gk, Gk);
            Se = fmaf(w, eps, Se);
            E0 = fmaf(w, coef0 * q0, E0);
            E1 = fmaf(w, fmaf(coef, q1, -G1), E1);
            E2 = fmaf(w, fmaf(coef, q2, -G2), E2);
            E3 = fmaf(w, fmaf(coef, q3, -G3), E3);
            S0 = fmaf(w, q0, S0); S1 = fmaf(w, q1, S1); S2 = fmaf(w, q2, S2); S3 = fmaf(w, q3, S3);
            SA = fmaf(w, u + wk + u * wk, SA);
            d0 = coef0 * k0;
            d1 = fmaf(coef, k1, -G1); d2 = fmaf(coef, k2, -G2); d3 = fmaf(coef, k3, -G3);
            dA = k0 * (adbf + dad);
            pk0 = k0; pk1 = k1; pk2 = k2; pk3 = k3;
        }
        {
            const double dl6 = dl * (1.0 / 6.0), dlL6 = dlL * (1.0 / 6.0);
            const float dl6f = (float)dl6, dlL6f = (float)dlL6;
            const double h6 = hubb * (6.0 + (double)Se);
            const double cd = dl6 * ((double)Gd - h6);
            p.k0 = fma(b.k0, dl6 * (-h6 - (double)Gk), b.k0 + (double)(dl6f * E0));
            p.k1 = fma(b.k1, cd, b.k1 + (double)(dl6f * E1));
            p.k2 = fma(b.k2, cd, b.k2 + (double)(dl6f * E2));
            p.k3 = fma(b.k3, cd, b.k3 + (double)(dl6f * E3));
            p.x = fma(dlL, b.k1, b.x + (double)(dlL6f * S1));
            p.y = fma(dlL, b.k2, b.y + (double)(dlL6f * S2));
            p.z = fma(dlL, b.k3, b.z + (double)(dlL6f * S3));
            p.t = fma(dl, b.k0, b.t + (double)(dl6f * S0));
            const double da = dl * b.k0 * adb;
            p.a = fma(da, (double)(SA * (1.f / 6.f)), b.a + da);
            // the step's displacement and conformal-time increment in FP32
            // (path length s and the ISW integral)
            const float ex = fmaf(dlLf, kb1, dlL6f * S1), ey = fmaf(dlLf, kb2, dlL6f * S2), ez = fmaf(dlLf, kb3, dlL6f * S3);
            sacc += (double)sqrtf(ex * ex + ey * ey + ez * ez);
            dtf = fmaf(dlf, kb0, dl6f * S0);
        }
        const Loc ploc = locate_near(T, here, p.x, p.y, p.z);
        data = born ? hom : gather_at<ORDER, VEL>(T, ploc, PosAt{p.x, p.y, p.z}, true, st, ST_POST_REC, false, vv);
        {
            // the extent test (integrator.h:757): a point in a located cell away from
            // the domain faces is inside; only cells on a face (or wrapped keys)
            // need the float64 comparison
            const uint32_t last = (ploc.cell >= 0) ? (uint32_t)((1ull << ploc.level) - 1ull) : 0u;
            const bool face = (ploc.cell < 0) || ploc.c[0] == 0u || ploc.c[1] == 0u || ploc.c[2] == 0u ||
                              ploc.c[0] >= last || ploc.c[1] >= last || ploc.c[2] >= last;
            if (p.a < 0.0 || (face && !((p.x > mn) && (p.x < mx) && (p.y > mn) && (p.y < mx) && (p.z > mn) && (p.z < mx)))) {
                clear(data);
                if (VEL) vv[0] = vv[1] = vv[2] = 0.f;
            }
        }
        if (VEL) p.dop = ((double)vv[0] * p.k1 + (double)vv[1] * p.k2 + (double)vv[2] * p.k3) / (kC * p.k0);
        p.level = (ploc.cell >= 0) ? ploc.level : 0;
        p.ah = data.a;
        p.rho = data.rho; p.phi = data.phi; p.dx = data.dx; p.dy = data.dy; p.dz = data.dz;
        p.dt = -data.dt;
        const float dphi_last = data.phi - (float)b.phi;   // laplacian of the final record, divided at the end
        const double dl_last = dl;
        isw += (double)((b.dt + p.dt) * dtf * inv_c2f);
        if (O.final_rec) {   // only the final photon record reports it
            iswold -= 2.0 * (p.phi - b.phi) * (1.0 / c2) -
                      (((double)b.dx + (double)p.dx) * (p.x - b.x) * scale + ((double)b.dy + (double)p.dy) * (p.y - b.y) * scale +
                       ((double)b.dz + (double)p.dz) * (p.z - b.z) * scale) * (1.0 / c2);
        }
        p.chi = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        lambda += dl;
        p.isw = isw; p.iswold = iswold; p.lambda = lambda; p.s = sacc;
        bool p_red_ok = false;
        auto need_p_red = [&]() { if (!p_red_ok) { p.red = red_of(p); p_red_ok = true; } };
        auto need_b_red = [&]() { if (!b_red_ok) { b.red = red_of(b); b_red_ok = true; } };
        if (!empty()) {
            const double ratio = p.a * p.a * ratio_k;
            dl = (ploc.cell >= 0 ? cell_extent(ploc.level) : 0.0) * ratio;
            last_data_dt = data.dt;
            last_dphi = dphi_last;
            last_dl = dl_last;
            if (ploc.cell != here.cell) stat(st, ST_CELL_CHANGE);
            here = ploc;
            ++k;
            stat(st, ST_STEPS);
            if (P.jacobian) {
                float h3[3];
                jac_fast(T, here, p.x, p.y, p.z, h3, st);
                const float dr = (float)(p.chi - b.chi), chif = (float)p.chi;
                chim2 = chim1; chim1 = b.chi;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    J.ckm1(q) = J.ck(q); J.ckm1(3 + q) = J.ck(3 + q);
                    const float c1 = chif * (h3[q] * dr), c2v = chif * c1;
                    J.ck(q) = c1;
                    J.ck(3 + q) = c2v;
                    J.S(q) += (double)c1;
                    J.S(3 + q) += (double)c2v;
                }
            }
            while (next_plane < np) {
                const int kind = skind;
                const double* kj = (WIDE && rki && kind == STOP_PLANE) ? rki + 3 * next_plane : nullptr;
                const double ref = SRC ? stop_ref : rpl[next_plane];
                bool crossed;
                if (!kj && kind == STOP_REDSHIFT) {
                    crossed = red_above(p, ref);
                } else {
                    const double q1 = kj ? (p.x * kj[0] + p.y * kj[1] + p.z * kj[2])
                                    : (kind == STOP_R) ? p.chi : (kind == STOP_LAMBDA) ? p.lambda : (kind == STOP_T) ? p.t
                                    : (kind == STOP_A) ? p.a : (kind == STOP_S) ? p.s : (need_p_red(), p.red);
                    crossed = (kind == STOP_A) ? (q1 < ref) : (q1 > ref);
                }
                if (!crossed) break;
                const int j = next_plane++;
                cross_k[j] = k;
                if (prow) {
                    need_p_red();
                    need_b_red();
                    double* o = prow + j * rec_fields;
                    const double q1 = kj ? (p.x * kj[0] + p.y * kj[1] + p.z * kj[2])
                                    : (kind == STOP_R) ? p.chi : (kind == STOP_LAMBDA) ? p.lambda : (kind == STOP_T) ? p.t
                                    : (kind == STOP_A) ? p.a : (kind == STOP_S) ? p.s : p.red;
                    const double q0 = kj ? (b.x * kj[0] + b.y * kj[1] + b.z * kj[2])
                                    : (kind == STOP_R) ? b.chi : (kind == STOP_LAMBDA) ? b.lambda : (kind == STOP_T) ? b.t
                                    : (kind == STOP_A) ? b.a : (kind == STOP_S) ? b.s : b.red;
                    const double f = (q1 - ref) / (q1 - q0);
                    const double px = b.x * f + p.x * (1 - f), py = b.y * f + p.y * (1 - f), pz = b.z * f + p.z * (1 - f);
                    const double dist = sqrt(px * px + py * py + pz * pz);
                    o[0] = (double)(k - 1); o[1] = f; o[2] = px; o[3] = py; o[4] = pz; o[5] = dist;
                    o[9] = b.t * f + p.t * (1 - f);
                    o[10] = b.a * f + p.a * (1 - f);
                    o[11] = b.red * f + p.red * (1 - f);
                    o[12] = b.chi * f + p.chi * (1 - f);
                    o[13] = b.lambda * f + p.lambda * (1 - f);
                    o[14] = b.s * f + p.s * (1 - f);
                    o[15] = b.isw * f + p.isw * (1 - f);
                    o[16] = (double)b.rho * f + (double)p.rho * (1 - f);
                    o[17] = b.phi * f + p.phi * (1 - f);
                    o[18] = have_rmax ? rmax : 0.0;
                    o[19] = 1.0;
                    if (SRC || WIDE) {
                        o[20] = b.k0 * f + p.k0 * (1 - f);
                        o[21] = b.k1 * f + p.k1 * (1 - f);
                        o[22] = b.k2 * f + p.k2 * (1 - f);
                        o[23] = b.k3 * f + p.k3 * (1 - f);
                    }
                    if (P.jacobian) {
                        // at the surface's distance, or at the source radius in source
                        // mode, or at the surface radius itself for a Born ray
                        const double jd = (SRC || born) ? ref : dist;
                        double s1[3], s2[3];
                        bool ok = true;
                        if (p.chi <= jd) {
                            for (int q = 0; q < 3; ++q) { s1[q] = J.S(q); s2[q] = J.S(3 + q); }
                        } else if (chim1 <= jd) {
                            for (int q = 0; q < 3; ++q) { s1[q] = J.S(q) - (double)J.ck(q); s2[q] = J.S(3 + q) - (double)J.ck(3 + q); }
                        } else if (k >= 2 && chim2 <= jd) {
                            for (int q = 0; q < 3; ++q) {
                                s1[q] = J.S(q) - (double)J.ck(q) - (double)J.ckm1(q);
                                s2[q] = J.S(3 + q) - (double)J.ck(3 + q) - (double)J.ckm1(3 + q);
                            }
                        } else {
                            ok = false;
                            status |= 2u;
                        }
                        if (ok) {
                            const double idist = 1.0 / jd;
                            o[6] = 1.0 - 2.0 * (s1[0] - s2[0] * idist) / c2 * P.length;
                            o[7] = -2.0 * (s1[1] - s2[1] * idist) / c2 * P.length;
                            o[8] = 1.0 - 2.0 * (s1[2] - s2[2] * idist) / c2 * P.length;
                        } else {
                            o[6] = 1.0; o[7] = 0.0; o[8] = 1.0;
                        }
                    } else {
                        o[6] = o[7] = o[8] = 0.0;
                    }
                }
            }
            if (!have_rmax || rmax < (double)b.rho) rmax = b.rho;
            have_rmax = true;
            b = p;
            b_red_ok = p_red_ok;
            if (WIDE && traj) {
                need_b_red();
                if (k < O.traj_cap) write_rec(traj + k * kPhotonFields, fast_record(b, last_data_dt, (double)last_dphi / last_dl, k));
                else status |= 8u;
            }
        }
        bool stop;
        switch (skind) {
        case STOP_R: stop = b.chi > stop_ref; break;
        case STOP_LAMBDA: stop = b.lambda > stop_ref; break;
        case STOP_REDSHIFT: stop = b_red_ok ? (b.red > stop_ref) : red_above(b, stop_ref); break;
        case STOP_T: stop = b.t > stop_ref; break;
        case STOP_A: stop = b.a < stop_ref; break;
        case STOP_PLANE: {
            const double* kk = (WIDE && rki) ? rki + 3 * (np - 1) : P.ki;
            stop = (p.x * kk[0] + p.y * kk[1] + p.z * kk[2]) > stop_ref;
            break;
        }
        case STOP_S: stop = b.s > stop_ref; break;
        default: stop = true;
        }
        if (stop) break;
    }
    if (!b_red_ok) b.red = red_of(b);
    long long size = k + 1;
    if (signbit(b.red) || signbit(b.a)) size -= 1;
    O.steps[i] = size;
    if (O.final_rec) {
        double* o = O.final_rec + i * kPhotonFields;
        if (size == k + 1) {
            write_rec(o, fast_record(b, last_data_dt, (double)last_dphi / last_dl, k));
        } else {
            for (int q = 0; q < kPhotonFields; ++q) o[q] = 0.0;
            status |= 4u;
        }
    }
    if (SRC && prow) {
        const long long ck = cross_k[0];
        const bool ok = (ck >= 1) && (ck < size);
        if (!ok) {
            for (int q = 0; q < 24; ++q) prow[q] = 0.0;
            const long long marked = size - 1;
            prow[0] = (double)(marked - (marked > 0));
            if (born && P.jacobian && ck < 0) {
                // a Born ray that ends short of the radius: the Jacobian at its last point
                const double idist = 1.0 / stop_ref;
                prow[6] = 1.0 - 2.0 * (J.S(0) - J.S(3) * idist) / c2 * P.length;
                prow[7] = -2.0 * (J.S(1) - J.S(4) * idist) / c2 * P.length;
                prow[8] = 1.0 - 2.0 * (J.S(2) - J.S(5) * idist) / c2 * P.length;
            }
        }
        prow[19] = ok ? 1.0 : 0.0;
    } else if (prow) {
        for (int j = 0; j < np; ++j) {
            double* o = prow + j * rec_fields;
            const long long ck = cross_k[j];
            const bool found = (ck >= 1) && (ck < size);
            const bool valid = found && !((ck - 1) == size - 1 || (ck - 1) == 0);
            if (ck < 0 || ck == 0 || ck >= size) {
                for (int q = 0; q < (WIDE ? 24 : kPlaneFields); ++q) o[q] = 0.0;
                o[0] = (ck == 0) ? 0.0 : (double)(size - 1);
            }
            o[19] = valid ? 1.0 : 0.0;
            if (WIDE) o[24] = found ? 1.0 : 0.0;
            if (born) {
                // Born ray (hmaps.h:712, 719): the Jacobian at the surface radius,
                // from the last point when the ray never got there; only a ray
                // that could not take a step is unusable
                if (P.jacobian && ck < 0) {
                    const double idist = 1.0 / rpl[j];
                    o[6] = 1.0 - 2.0 * (J.S(0) - J.S(3) * idist) / c2 * P.length;
                    o[7] = -2.0 * (J.S(1) - J.S(4) * idist) / c2 * P.length;
                    o[8] = 1.0 - 2.0 * (J.S(2) - J.S(5) * idist) / c2 * P.length;
                }
                o[19] = (size > 1) ? 1.0 : 0.0;
            }
        }
    }
    if (status) atomicOr(O.status, status);
}


// Persistent launch: each warp takes the next 32 x depth rays of [lo, n) from
// a global counter until the range is exhausted, so uneven path lengths do
// not leave tail waves; its lanes trace them depth at a time.  `queue` is
// zeroed before the launch.  The block size and depth are the autotuner's
// (mpf_prop_fast.cu); the rays' results do not depend on them.
#if defined(MPF_FAST_MAXNREG)
#define MPF_FAST_BOUNDS __maxnreg__(MPF_FAST_MAXNREG)
#else
#define MPF_FAST_BOUNDS __launch_bounds__(kFastThreads, MPF_FAST_MINB)
#endif
template <int ORDER, bool SRC, bool WIDE, bool BORN = false, bool VEL = false>
__global__ void MPF_FAST_BOUNDS k_propagate_fast(DevTree T, DevCosmo C, PropParams P,
                                                                    const double* __restrict__ launch, long long n, PropOut O,
                                                                    unsigned long long* queue, int depth, long long lo)
{
    __shared__ double jac_sums[6 * kFastThreads];
    __shared__ float jac_terms[12 * kFastThreads];
    const JacSums J{jac_sums + threadIdx.x, jac_terms + threadIdx.x};
    const int lane = threadIdx.x & 31;
    const unsigned long long per = 32ull * (unsigned long long)depth;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(queue, per);
        base = __shfl_sync(0xffffffffu, base, 0) + (unsigned long long)lo;
        if (base >= (unsigned long long)n) break;
        for (int d = 0; d < depth; ++d) {
            const long long i = (long long)base + 32ll * d + lane;
            if (i < n) propagate_fast<ORDER, SRC, WIDE, BORN, VEL>(T, C, P, launch + 6 * i, i, O, J);
            __syncwarp();
        }
    }
}

// Fast-mode gathers through the stencil records (tests / mpf_interpolate).
static __global__ void k_gather_rec(DevTree T, int kind, const double* __restrict__ xyz, long long n, void* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    const Loc d = locate_full(T, x, y, z);
    if (kind == 0) {
        ((long long*)out)[i] = d.cell;
        return;
    }
    const Field7 f = (kind == 1) ? gather_at<1>(T, d, PosAt{x, y, z}, true, nullptr, 0, true)
                                 : gather_at<2>(T, d, PosAt{x, y, z}, true, nullptr, 0, true);
    float* o = (float*)out + 7 * i;
    o[0] = f.rho; o[1] = f.phi; o[2] = f.dx; o[3] = f.dy; o[4] = f.dz; o[5] = f.a; o[6] = f.dt;
}

}  // namespace mpf
