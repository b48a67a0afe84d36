// Device-side octree lookups and the CIC / TSC gathers.
//
// Layout in HBM (built by mpf_octree.cu):
//   keys[n]      ulonglong2 (hi, lo), sorted: cell index == the reference's
//                iterator position in its sorted container
//   grad[n]      float4 (dphidx, dphidy, dphidz, dphidt) per cell
//   scal[n]      float4 (rho, phi, a, level as int bits) per cell
//   node[m]      int2 (first child node or -1, cell index or -1); nodes are
//                level-ordered and a refined node's 8 children are
//                contiguous in site order (site = x | y<<1 | z<<2)
//   grid[gx*gy*gz] int32 node index of each level-Lt cell of the bounding box
//   vel[n]       float4 (vx, vy, vz, 0) per cell, in units of c: the velocity
//                slots of the velocity-field octree (gravity2.h:45), or absent
//
// find_cell() returns what the reference's
//   upper_bound(keys, K) - 1, if that key contains K          (simplehyperoctree.h:874-899)
// returns, for the level-L key K with integer coordinates (cx, cy, cz): the
// deepest existing cell containing K, provided no existing key lies strictly
// between it and K (checked against the next sorted key only when that cell
// has descendants; otherwise it is implied by pre-order sorting).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mpf_keys.cuh"

namespace mpf {

struct DevTree {
    const ulonglong2* keys;
    const float4* grad;
    const float4* scal;
    const int2* node;
    const int* grid;
    // per-cell stencil records, 8 x int4 (128 B) per cell:
    //   ints 0..26  the 27 cells of the cell's level around it, x-major
    //               (ix outer, iz inner), each the reference lookup result
    //               (deepest existing cell <= that level, or -1)
    //   int 27      level | has_children << 8
    //   int 28      bit j set: entry j is at exactly the cell's level
    //   int 29      node index of the cell
    //   int 30      the parent cell (one level up), or -1
    const int4* stencil;
    // per-cell velocity (vx, vy, vz, 0), or null: an octree without a
    // velocity field (the reference built without -DVELOCITYFIELD)
    const float4* vel;
    int64_t n;
    int Lt;                // level of the top grid
    int gx0, gy0, gz0;     // grid origin (integer coords at Lt)
    int gnx, gny, gnz;     // grid dims
};

struct Found {
    int cell;   // -1 if not found
    int level;
};

__device__ __forceinline__ Found find_cell(const DevTree& T, int L, uint64_t cx, uint64_t cy, uint64_t cz)
{
    Found r{-1, 0};
    if (L < T.Lt) return r;
    const int sh = L - T.Lt;
    const long gx = (long)(cx >> sh) - T.gx0, gy = (long)(cy >> sh) - T.gy0, gz = (long)(cz >> sh) - T.gz0;
    if (gx < 0 || gy < 0 || gz < 0 || gx >= T.gnx || gy >= T.gny || gz >= T.gnz) return r;
    int nd = __ldg(T.grid + ((gz * T.gny + gy) * (long)T.gnx + gx));
    if (nd < 0) return r;
    int2 cur = __ldg(T.node + nd);
    int bnode = nd, bl = T.Lt;
    r.cell = cur.y;
    for (int l = T.Lt + 1; l <= L && cur.x >= 0; ++l) {
        const int b = L - l;
        const int site = (int)((cx >> b) & 1ull) | ((int)((cy >> b) & 1ull) << 1) | ((int)((cz >> b) & 1ull) << 2);
        nd = cur.x + site;
        cur = __ldg(T.node + nd);
        if (cur.y >= 0) { r.cell = cur.y; bnode = nd; bl = l; }
    }
    if (r.cell < 0) return r;
    r.level = bl;
    if (bl < L && __ldg(&T.node[bnode].x) >= 0 && r.cell + 1 < T.n) {
        // the found cell has descendants: make sure none of them precedes K
        const ulonglong2 nk = __ldg(T.keys + r.cell + 1);
        const Key K = key_from_coords(L, cx, cy, cz);
        if (key_le(Key{nk.x, nk.y}, K)) r.cell = -1;
    }
    return r;
}

// 7-field record in the reference's Gravity order.
struct Field7 {
    float rho, phi, dx, dy, dz, a, dt;
};

__device__ __forceinline__ void clear(Field7& f) { f = Field7{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}; }
__device__ __forceinline__ bool is_empty(const Field7& f)
{
    return f.rho == 0.f && f.phi == 0.f && f.dx == 0.f && f.dy == 0.f && f.dz == 0.f && f.a == 0.f && f.dt == 0.f;
}

// acc += v * w with the reference's rounding: (float)((double)acc + (double)v * w)
__device__ __forceinline__ float mac64(float acc, float v, double w)
{
    return __double2float_rn(__dadd_rn((double)acc, __dmul_rn((double)v, w)));
}

template <bool EXACT>
__device__ __forceinline__ void mac_cell(const DevTree& T, Field7& acc, int cell, double w, bool need_all)
{
    const float4 g = __ldg(T.grad + cell);
    if (EXACT) {
        acc.dx = mac64(acc.dx, g.x, w);
        acc.dy = mac64(acc.dy, g.y, w);
        acc.dz = mac64(acc.dz, g.z, w);
        acc.dt = mac64(acc.dt, g.w, w);
        if (need_all) {
            const float4 s = __ldg(T.scal + cell);
            acc.rho = mac64(acc.rho, s.x, w);
            acc.phi = mac64(acc.phi, s.y, w);
            acc.a = mac64(acc.a, s.z, w);
        }
    } else {
        const float wf = (float)w;
        acc.dx = fmaf(g.x, wf, acc.dx);
        acc.dy = fmaf(g.y, wf, acc.dy);
        acc.dz = fmaf(g.z, wf, acc.dz);
        acc.dt = fmaf(g.w, wf, acc.dt);
        if (need_all) {
            const float4 s = __ldg(T.scal + cell);
            acc.rho = fmaf(s.x, wf, acc.rho);
            acc.phi = fmaf(s.y, wf, acc.phi);
            acc.a = fmaf(s.z, wf, acc.a);
        }
    }
}

// Accumulator of the CIC / TSC walks: the 7 Gravity fields and, with V, the
// velocity slots of the velocity-field octree (gravity2.h:45), which the
// reference's multiply-accumulate treats like the other fields
// (simplehyperoctree.h:1887-1910: every arithmetic member of the record, with
// the same weight and rounding).
template <bool V>
struct GatherAcc {
    Field7 f;
    float v[3];
    bool need_all;
    __device__ __forceinline__ void reset()
    {
        clear(f);
        if (V) v[0] = v[1] = v[2] = 0.f;
    }
    template <bool EXACT>
    __device__ __forceinline__ void add(const DevTree& T, int cell, double w)
    {
        mac_cell<EXACT>(T, f, cell, w, need_all);
        if (V) {
            const float4 u = __ldg(T.vel + cell);
            if (EXACT) {
                v[0] = mac64(v[0], u.x, w);
                v[1] = mac64(v[1], u.y, w);
                v[2] = mac64(v[2], u.z, w);
            } else {
                const float wf = (float)w;
                v[0] = fmaf(u.x, wf, v[0]);
                v[1] = fmaf(u.y, wf, v[1]);
                v[2] = fmaf(u.z, wf, v[2]);
            }
        }
    }
};

// Deepest cell at the position (reference locate()); -1 if none.
__device__ __forceinline__ Found locate(const DevTree& T, double x, double y, double z)
{
    return find_cell(T, kMaxLevel, axis_coord(kMaxLevel, x), axis_coord(kMaxLevel, y), axis_coord(kMaxLevel, z));
}

// find_cell(T, L, k) for the integer coordinates k of a level-L key, read
// from the stencil record of the level-L cell `centre` (coordinates cc) when
// k is one of its 27 neighbours (the record holds find_cell's result for each
// of them), else found by the walk.  centre < 0: no record to read.
#ifndef MPF_EXACT_STENCIL
#define MPF_EXACT_STENCIL 1
#endif
__device__ __forceinline__ Found find_near(const DevTree& T, int centre, int L, const uint64_t* cc, const uint64_t* k)
{
    if (MPF_EXACT_STENCIL && centre >= 0 && L >= 2) {
        const uint64_t mask = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);
        int o[3];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const uint64_t dm = (k[d] - cc[d]) & mask;
            o[d] = (dm == 0) ? 0 : (dm == 1) ? 1 : (dm == mask) ? -1 : 2;
            ok = ok && o[d] != 2;
        }
        if (ok) {
            const int e = __ldg(reinterpret_cast<const int*>(T.stencil + 8 * (size_t)centre) + (o[0] + 1) * 9 +
                                (o[1] + 1) * 3 + (o[2] + 1));
            if (e < 0) return Found{-1, 0};
            return Found{e, __float_as_int(__ldg(&T.scal[e].w))};
        }
    }
    return find_cell(T, L, k[0], k[1], k[2]);
}

// the level-`to` ancestor of the level-`from` cell `cell` through the records'
// parent links, or -1
__device__ __forceinline__ int ancestor_cell(const DevTree& T, int cell, int from, int to)
{
    for (int l = from; l > to && cell >= 0; --l)
        cell = __ldg(reinterpret_cast<const int*>(T.stencil + 8 * (size_t)cell) + 30);
    return cell;
}

// Cloud-in-cell (simplehyperoctree.h:1410-1469): trilinear over the 8 cells
// of the located cell's level; restarts one level up when a neighbour is
// coarser; empty when a neighbour is missing.  res.need_all = also accumulate
// rho, phi, a (the RK stages only need the gradient and dphidt).
template <bool EXACT, bool V>
__device__ void cic_walk(const DevTree& T, double x, double y, double z, GatherAcc<V>& res)
{
    res.reset();
    const uint64_t c32x = axis_coord(kMaxLevel, x), c32y = axis_coord(kMaxLevel, y), c32z = axis_coord(kMaxLevel, z);
    const Found f0 = find_cell(T, kMaxLevel, c32x, c32y, c32z);
    if (f0.cell < 0) return;
    int ilvl = f0.level, lvl = ilvl;
    // coordinates of the current centre cell at level ilvl (and, exact mode, its
    // record: the vertex lookups read it)
    uint64_t ccx = c32x >> (kMaxLevel - ilvl), ccy = c32y >> (kMaxLevel - ilvl), ccz = c32z >> (kMaxLevel - ilvl);
    int centre = f0.cell;
    // the child site holding the point: next bit below the centre's level
    int site = 0;
    if (ilvl < kMaxLevel) {
        const int b = kMaxLevel - ilvl - 1;
        site = (int)((c32x >> b) & 1ull) | ((int)((c32y >> b) & 1ull) << 1) | ((int)((c32z >> b) & 1ull) << 2);
    }
    double half = half_cell(ilvl);
    const double pt[3] = {x, y, z};
    do {
        ilvl = lvl;
        const double cen[3] = {coord_center(ilvl, ccx), coord_center(ilvl, ccy), coord_center(ilvl, ccz)};
        double dist[3];
        for (int d = 0; d < 3; ++d) dist[d] = fabs(__ddiv_rn(__dsub_rn(cen[d], pt[d]), __dadd_rn(half, half)));
        for (int v = 0; v < 8; ++v) {
            double w = 1.0;
            const int diff = site ^ v;
            uint64_t kc[3];
            for (int d = 0; d < 3; ++d) {
                const int bb = (v >> d) & 1, db = (diff >> d) & 1;
                double vert;
                if (EXACT) {
                    vert = __dsub_rn(__dadd_rn(pt[d], __dmul_rn((double)bb, half)), __dmul_rn((double)(!bb), half));
                    w = __dmul_rn(w, __dadd_rn(__dmul_rn((double)db, __dsub_rn(1.0, dist[d])), __dmul_rn((double)(!db), dist[d])));
                    kc[d] = axis_coord(ilvl, vert);
                } else {
                    w *= db ? (1.0 - dist[d]) : dist[d];
                    const uint64_t c = (d == 0) ? ccx : ((d == 1) ? ccy : ccz);
                    const int sbit = (site >> d) & 1;
                    // the vertex cell is the centre cell, or its neighbour on the point's side
                    kc[d] = (c + (uint64_t)(bb + sbit) - 1ull) & ((1ull << ilvl) - 1ull);
                    (void)vert;
                }
            }
            const uint64_t cc[3] = {ccx, ccy, ccz};
            const Found fi = EXACT ? find_near(T, centre, ilvl, cc, kc) : find_cell(T, ilvl, kc[0], kc[1], kc[2]);
            if (fi.cell >= 0) {
                lvl = min(lvl, fi.level);
                res.template add<EXACT>(T, fi.cell, w);
            } else {
                res.reset();
                break;
            }
        }
        if (lvl < ilvl) {
            // restart on the level-lvl cell containing the point
            const int b = kMaxLevel - (lvl + 1);
            const uint64_t px = c32x >> b, py = c32y >> b, pz = c32z >> b;   // coords at lvl+1
            site = (int)(px & 1ull) | ((int)(py & 1ull) << 1) | ((int)(pz & 1ull) << 2);
            ccx = px >> 1; ccy = py >> 1; ccz = pz >> 1;
            if (EXACT) centre = ancestor_cell(T, centre, ilvl, lvl);
            res.reset();
            half = half_cell(lvl);
        }
    } while (lvl < ilvl);
}

template <bool EXACT>
__device__ Field7 cic(const DevTree& T, double x, double y, double z, bool need_all)
{
    GatherAcc<false> res;
    res.need_all = need_all;
    cic_walk<EXACT, false>(T, x, y, z, res);
    return res.f;
}

__device__ __forceinline__ double tsc_w1(int a, double d)
{
    // (a*0.5*(1.5-d)*(1.5-d) + (1-a)*(0.75-d*d)), left to right, no contraction
    const double t1 = __dmul_rn(__dmul_rn(__dmul_rn((double)a, 0.5), __dsub_rn(1.5, d)), __dsub_rn(1.5, d));
    const double t2 = __dmul_rn((double)(1 - a), __dsub_rn(0.75, __dmul_rn(d, d)));
    return __dadd_rn(t1, t2);
}

__device__ __forceinline__ float tsc_w1f(int a, float d)
{
    return a ? 0.5f * (1.5f - d) * (1.5f - d) : 0.75f - d * d;
}

// Triangular-shaped cloud (simplehyperoctree.h:1479-1644): quadratic weights
// over the 27 cells of the located cell's level, x-major (ix, iy, iz) order;
// restarts at the level of the first coarser neighbour; empty when one is
// missing; CIC at the exact origin.
template <bool EXACT, bool V>
__device__ void tsc_walk(const DevTree& T, double x, double y, double z, GatherAcc<V>& res)
{
    if (x == 0.0 && y == 0.0 && z == 0.0) {
        cic_walk<EXACT, V>(T, 0., 0., 0., res);
        return;
    }
    res.reset();
    const uint64_t c32x = axis_coord(kMaxLevel, x), c32y = axis_coord(kMaxLevel, y), c32z = axis_coord(kMaxLevel, z);
    const Found f0 = find_cell(T, kMaxLevel, c32x, c32y, c32z);
    if (f0.cell < 0) return;
    int ilvl = f0.level, lvl = ilvl;
    int centre = f0.cell;   // the record of the centre cell at level ilvl (exact mode)
    double half = half_cell(ilvl);
    const double pt[3] = {x, y, z};
    do {
        if (EXACT && lvl < ilvl) centre = ancestor_cell(T, centre, ilvl, lvl);
        ilvl = lvl;
        const double tw = __dmul_rn(2.0, half);
        const uint64_t ccx = c32x >> (kMaxLevel - ilvl), ccy = c32y >> (kMaxLevel - ilvl), ccz = c32z >> (kMaxLevel - ilvl);
        bool stop = false;
        // fast mode: fractional offsets of the point from the centre cell, shared by all 27 weights
        float fd[3];
        if (!EXACT) {
            const double cx = coord_center(ilvl, ccx), cy = coord_center(ilvl, ccy), cz = coord_center(ilvl, ccz);
            fd[0] = (float)((x - cx) / tw);
            fd[1] = (float)((y - cy) / tw);
            fd[2] = (float)((z - cz) / tw);
        }
        for (int ix = -1; ix <= 1 && !stop; ++ix) {
            for (int iy = -1; iy <= 1 && !stop; ++iy) {
                for (int iz = -1; iz <= 1 && !stop; ++iz) {
                    uint64_t kx, ky, kz;
                    double w;
                    if (EXACT) {
                        const double qx = __dadd_rn(pt[0], __dmul_rn((double)ix, tw));
                        const double qy = __dadd_rn(pt[1], __dmul_rn((double)iy, tw));
                        const double qz = __dadd_rn(pt[2], __dmul_rn((double)iz, tw));
                        kx = axis_coord(ilvl, qx);
                        ky = axis_coord(ilvl, qy);
                        kz = axis_coord(ilvl, qz);
                        const double d0 = fabs(__ddiv_rn(__dsub_rn(coord_center(ilvl, kx), pt[0]), tw));
                        const double d1 = fabs(__ddiv_rn(__dsub_rn(coord_center(ilvl, ky), pt[1]), tw));
                        const double d2 = fabs(__ddiv_rn(__dsub_rn(coord_center(ilvl, kz), pt[2]), tw));
                        w = __dmul_rn(__dmul_rn(tsc_w1(abs(ix), d0), tsc_w1(abs(iy), d1)), tsc_w1(abs(iz), d2));
                    } else {
                        const uint64_t m = (1ull << ilvl) - 1ull;
                        kx = (ccx + (uint64_t)(int64_t)ix) & m;
                        ky = (ccy + (uint64_t)(int64_t)iy) & m;
                        kz = (ccz + (uint64_t)(int64_t)iz) & m;
                        const float wf = tsc_w1f(abs(ix), fabsf(fd[0] - (float)ix)) * tsc_w1f(abs(iy), fabsf(fd[1] - (float)iy)) *
                                         tsc_w1f(abs(iz), fabsf(fd[2] - (float)iz));
                        w = (double)wf;
                    }
                    const uint64_t kk[3] = {kx, ky, kz}, cc[3] = {ccx, ccy, ccz};
                    const Found fi = EXACT ? find_near(T, centre, ilvl, cc, kk) : find_cell(T, ilvl, kx, ky, kz);
                    if (fi.cell >= 0) {
                        lvl = min(lvl, fi.level);
                        if (lvl < ilvl) { res.reset(); stop = true; }
                        else res.template add<EXACT>(T, fi.cell, w);
                    } else {
                        res.reset();
                        stop = true;
                    }
                }
            }
        }
        if (lvl < ilvl) {
            res.reset();
            half = half_cell(lvl);
        }
    } while (lvl < ilvl);
}

template <bool EXACT>
__device__ Field7 tsc(const DevTree& T, double x, double y, double z, bool need_all)
{
    GatherAcc<false> res;
    res.need_all = need_all;
    tsc_walk<EXACT, false>(T, x, y, z, res);
    return res.f;
}

// Nearest grid point (simplehyperoctree.h:1396-1401): the data of the
// deepest cell containing the position, or the empty record.
__device__ __forceinline__ Field7 ngp(const DevTree& T, double x, double y, double z)
{
    Field7 f;
    clear(f);
    const Found c = locate(T, x, y, z);
    if (c.cell < 0) return f;
    const float4 g = __ldg(T.grad + c.cell);
    const float4 s = __ldg(T.scal + c.cell);
    f.rho = s.x; f.phi = s.y; f.a = s.z;
    f.dx = g.x; f.dy = g.y; f.dz = g.z; f.dt = g.w;
    return f;
}

template <bool EXACT>
__device__ __forceinline__ Field7 gather(const DevTree& T, int order, double x, double y, double z, bool need_all)
{
    if (order == 0) return ngp(T, x, y, z);
    return (order == 1) ? cic<EXACT>(T, x, y, z, need_all) : tsc<EXACT>(T, x, y, z, need_all);
}

// The 7 fields and the velocity v[3] at a point of a velocity-field octree
// (T.vel set), through the same cells and weights.
template <bool EXACT>
__device__ Field7 gather_vel(const DevTree& T, int order, double x, double y, double z, float* v)
{
    if (order == 0) {
        const Found c = locate(T, x, y, z);
        const float4 u = (c.cell >= 0) ? __ldg(T.vel + c.cell) : make_float4(0.f, 0.f, 0.f, 0.f);
        v[0] = u.x; v[1] = u.y; v[2] = u.z;
        return ngp(T, x, y, z);
    }
    GatherAcc<true> res;
    res.need_all = true;
    if (order == 1) cic_walk<EXACT, true>(T, x, y, z, res);
    else tsc_walk<EXACT, true>(T, x, y, z, res);
    v[0] = res.v[0]; v[1] = res.v[1]; v[2] = res.v[2];
    return res.f;
}

}  // namespace mpf
