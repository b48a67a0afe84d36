// Throughput mode of the propagation kernel.
//
// Same algorithm as propagate_one<EXACT> (src/integrator.h:648-824 with the
// fused src/lensing.h:399-472 Jacobian), reorganised for the GB300's
// arithmetic balance:
//
//  * Cell window.  Each ray keeps, in shared memory, the cell indices of the
//    5x5x5 block of cells of its current level around the cell it is in,
//    each tagged "has children".  A TSC stencil whose 27 cells are all in the
//    window at that level, around a leaf centre, is gathered straight from the
//    window; anything else (refinement boundaries, missing or coarser
//    neighbours, the origin) falls back to the full lookup, which keeps the
//    reference's restart semantics.  The window is rebuilt when the ray
//    enters another cell (every ~8-30 steps), so the steady state does no
//    octree walks at all.
//  * The six Jacobian gathers at +-1 cell are the finite differences of TSC
//    sums over the 5x3x3 boxes of the window; they are evaluated as one sum
//    with the weight differences, which is the same quantity without the
//    cancellation of subtracting two TSC values.
//  * FP64 is kept for the RK4 state, the RHS, affine parameter, redshift and
//    distances.  Cell coordinates use exact power-of-two scalings (no
//    divisions), TSC weights and field accumulation are FP32, the cosmology
//    search uses a uniform index table.
#pragma once
#include "mpf_propagate.cuh"

namespace mpf {

constexpr int kWin = 5;
constexpr int kWin3 = kWin * kWin * kWin;
constexpr int kHasChildren = 1 << 30;
constexpr int kCellMask = kHasChildren - 1;

__device__ __forceinline__ int widx(int ox, int oy, int oz) { return ((oz + 2) * kWin + (oy + 2)) * kWin + (ox + 2); }

// Utility::interpolate with the uniform index table (same bracketing interval
// as the reference's upper_bound; slope precomputed per interval).
__device__ __forceinline__ double interp_fast(const DevCosmo& C, double x0, const double* __restrict__ y,
                                              const double* __restrict__ slope)
{
    int i;
    if (x0 < C.t0) {
        i = 0;
    } else {
        double kk = (x0 - C.t0) * C.lut_scale;
        int k = (kk < (double)C.nlut) ? (int)kk : C.nlut;
        i = __ldg(C.lut + k);
        while (i < C.n && !(x0 < __ldg(C.t + i))) ++i;
    }
    const int n = C.n;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n <= 1) return (n > 0) ? __ldg(y) : 0.0;
    return __ldg(y + i - 1) + __ldg(slope + i - 1) * (x0 - __ldg(C.t + i - 1));
}

struct Win {
    uint32_t cx, cy, cz;
    int level;        // -1: no window
    bool core_ok;     // the 27 cells around the centre exist at `level` and the centre is a leaf
    bool jac_ok;      // core_ok, the 81-cell cross exists, and the 6 face neighbours are leaves
};

// The 125 lookups advance together, one tree level per round, so each round
// is 125 independent loads instead of 125 dependent chains.  The shared-memory
// slots hold the running node index between rounds.
__device__ void win_build(const DevTree& T, int L, uint32_t cx, uint32_t cy, uint32_t cz, int* ws, int stride, Win& w)
{
    const uint64_t mask = (L >= 32) ? 0xffffffffull : ((1ull << L) - 1ull);
    const int sh = L - T.Lt;
    // round 0: top-grid entries
    for (int k = 0; k < kWin3; ++k) {
        const int ox = k % kWin - 2, oy = (k / kWin) % kWin - 2, oz = k / (kWin * kWin) - 2;
        const uint64_t qx = ((uint64_t)cx + (uint64_t)(int64_t)ox) & mask, qy = ((uint64_t)cy + (uint64_t)(int64_t)oy) & mask,
                       qz = ((uint64_t)cz + (uint64_t)(int64_t)oz) & mask;
        int nd = -1;
        if (sh >= 0) {
            const long gx = (long)(qx >> sh) - T.gx0, gy = (long)(qy >> sh) - T.gy0, gz = (long)(qz >> sh) - T.gz0;
            if (gx >= 0 && gy >= 0 && gz >= 0 && gx < T.gnx && gy < T.gny && gz < T.gnz)
                nd = __ldg(T.grid + ((gz * T.gny + gy) * (long)T.gnx + gx));
        }
        ws[k * stride] = nd;
    }
    // rounds 1..L-Lt: descend one level; a slot that cannot descend becomes -1
    for (int l = T.Lt + 1; l <= L; ++l) {
        const int b = L - l;
#pragma unroll 5
        for (int k = 0; k < kWin3; ++k) {
            int nd = ws[k * stride];
            if (nd >= 0) {
                const int child = __ldg(&T.node[nd].x);
                if (child < 0) nd = -1;
                else {
                    const int ox = k % kWin - 2, oy = (k / kWin) % kWin - 2, oz = k / (kWin * kWin) - 2;
                    const uint64_t qx = ((uint64_t)cx + (uint64_t)(int64_t)ox) & mask, qy = ((uint64_t)cy + (uint64_t)(int64_t)oy) & mask,
                                   qz = ((uint64_t)cz + (uint64_t)(int64_t)oz) & mask;
                    nd = child + ((int)((qx >> b) & 1ull) | ((int)((qy >> b) & 1ull) << 1) | ((int)((qz >> b) & 1ull) << 2));
                }
                ws[k * stride] = nd;
            }
        }
    }
    // last round: node -> tagged cell, and the window flags
    bool core = true, jac = true;
#pragma unroll 5
    for (int k = 0; k < kWin3; ++k) {
        const int nd = ws[k * stride];
        int e = -1;
        if (nd >= 0) {
            const int2 v = __ldg(T.node + nd);
            if (v.y >= 0) e = v.y | ((v.x >= 0) ? kHasChildren : 0);
        }
        ws[k * stride] = e;
        const int ox = k % kWin - 2, oy = (k / kWin) % kWin - 2, oz = k / (kWin * kWin) - 2;
        const int ax = abs(ox), ay = abs(oy), az = abs(oz);
        const bool inner = ax <= 1 && ay <= 1 && az <= 1;
        const bool cross = (ax <= 2 && ay <= 1 && az <= 1) || (ax <= 1 && ay <= 2 && az <= 1) || (ax <= 1 && ay <= 1 && az <= 2);
        if (inner && e < 0) core = false;
        if (cross && e < 0) jac = false;
        if ((ax + ay + az) <= 1 && (e < 0 || (e & kHasChildren))) {
            jac = false;
            if (ax + ay + az == 0) core = false;
        }
    }
    w.cx = cx; w.cy = cy; w.cz = cz; w.level = L;
    w.core_ok = core;
    w.jac_ok = core && jac;
}

// integer coordinates at level L and the offset of the point from its cell
// centre in cell units (exact scaling by 2^L / EXTENT)
__device__ __forceinline__ void point_cell(int L, double x, double y, double z, uint32_t* c, float* fd)
{
    const double s = (double)(1ull << L) * (1.0 / (double)kExtent);
    const double u[3] = {(x + 2.0) * s, (y + 2.0) * s, (z + 2.0) * s};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double f = floor(u[d]);
        c[d] = (f > 0.0) ? (uint32_t)(uint64_t)f : 0u;
        fd[d] = (float)(u[d] - f) - 0.5f;
    }
}

__device__ __forceinline__ void tsc_w3(float f, float* w)
{
    const float m = 0.5f - f, p = 0.5f + f;
    w[0] = 0.5f * m * m;
    w[1] = 0.75f - f * f;
    w[2] = 0.5f * p * p;
}

// TSC through the window; returns false (and leaves `res` untouched) when the
// stencil is not fully inside the window at the window's level.
__device__ __forceinline__ bool tsc_win(const DevTree& T, const Win& w, const int* ws, int stride, double x, double y, double z,
                                        bool need_all, Field7& res)
{
    if (w.level < 0) return false;
    if (x == 0.0 && y == 0.0 && z == 0.0) return false;
    uint32_t c[3];
    float fd[3];
    point_cell(w.level, x, y, z, c, fd);
    const int ox = (int)(c[0] - w.cx), oy = (int)(c[1] - w.cy), oz = (int)(c[2] - w.cz);
    if (abs(ox) > 1 || abs(oy) > 1 || abs(oz) > 1) return false;
    const int ec = ws[widx(ox, oy, oz) * stride];
    if (ec < 0 || (ec & kHasChildren)) return false;
    if (!(w.core_ok && ox == 0 && oy == 0 && oz == 0)) {
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                    if (ws[widx(ox + dx, oy + dy, oz + dz) * stride] < 0) return false;
    }
    float wx[3], wy[3], wz[3];
    tsc_w3(fd[0], wx);
    tsc_w3(fd[1], wy);
    tsc_w3(fd[2], wz);
    float gx = 0.f, gy = 0.f, gz = 0.f, gt = 0.f, rho = 0.f, phi = 0.f, a = 0.f;
    // x-major order as the reference (ix outermost)
#pragma unroll
    for (int ix = 0; ix < 3; ++ix) {
#pragma unroll
        for (int iy = 0; iy < 3; ++iy) {
            const float wxy = wx[ix] * wy[iy];
#pragma unroll
            for (int iz = 0; iz < 3; ++iz) {
                const float wt = wxy * wz[iz];
                const int cell = ws[widx(ox + ix - 1, oy + iy - 1, oz + iz - 1) * stride] & kCellMask;
                const float4 g = __ldg(T.grad + cell);
                gx = fmaf(g.x, wt, gx);
                gy = fmaf(g.y, wt, gy);
                gz = fmaf(g.z, wt, gz);
                gt = fmaf(g.w, wt, gt);
                if (need_all) {
                    const float4 s = __ldg(T.scal + cell);
                    rho = fmaf(s.x, wt, rho);
                    phi = fmaf(s.y, wt, phi);
                    a = fmaf(s.z, wt, a);
                }
            }
        }
    }
    res = Field7{rho, phi, gx, gy, gz, a, gt};
    return true;
}

// Hessian terms of the infinitesimal Jacobian (lensing.h:430-443) from the
// window: d_ij = [TSC(x + h e_j).dphidi - TSC(x - h e_j).dphidi] / (2h), h = one cell.
__device__ __forceinline__ void hessian_win(const DevTree& T, const int* ws, int stride, const float* fd, float inv_dl, float* H)
{
    float wx[3], wy[3], wz[3];
    tsc_w3(fd[0], wx);
    tsc_w3(fd[1], wy);
    tsc_w3(fd[2], wz);
    // weight differences over 5 cells: (+h stencil) - (-h stencil)
    const float dx5[5] = {-wx[0], -wx[1], wx[0] - wx[2], wx[1], wx[2]};
    const float dy5[5] = {-wy[0], -wy[1], wy[0] - wy[2], wy[1], wy[2]};
    const float dz5[5] = {-wz[0], -wz[1], wz[0] - wz[2], wz[1], wz[2]};
    float dxx = 0.f, dxy = 0.f, dyy = 0.f, dxz = 0.f, dyz = 0.f, dzz = 0.f;
    // x box: 5 x 3 x 3
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                const float4 g = __ldg(T.grad + (ws[widx(i - 2, j - 1, k - 1) * stride] & kCellMask));
                dxx = fmaf(g.x, dx5[i] * wy[j] * wz[k], dxx);
            }
    // y box
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 5; ++j)
            for (int k = 0; k < 3; ++k) {
                const float4 g = __ldg(T.grad + (ws[widx(i - 1, j - 2, k - 1) * stride] & kCellMask));
                const float wt = wx[i] * dy5[j] * wz[k];
                dxy = fmaf(g.x, wt, dxy);
                dyy = fmaf(g.y, wt, dyy);
            }
    // z box
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 5; ++k) {
                const float4 g = __ldg(T.grad + (ws[widx(i - 1, j - 1, k - 2) * stride] & kCellMask));
                const float wt = wx[i] * wy[j] * dz5[k];
                dxz = fmaf(g.x, wt, dxz);
                dyz = fmaf(g.y, wt, dyz);
                dzz = fmaf(g.z, wt, dzz);
            }
    H[0] = dxx * inv_dl; H[1] = dxy * inv_dl; H[2] = dxz * inv_dl;
    H[3] = dyy * inv_dl; H[4] = dyz * inv_dl; H[5] = dzz * inv_dl;
}

// Jacobian contribution (d1d1, d1d2, d2d2 of lensing.h:444-447) at point p
// whose deepest cell is the window centre (or a fallback to six full TSC).
__device__ __forceinline__ void jac_fast(const DevTree& T, const Win& w, const int* ws, int stride, double x, double y,
                                         double z, int level, float* out3)
{
    float H[6];
    const double dl = ldexp(1.0, kLevelShift + 1 - level);
    bool done = false;
    if (w.jac_ok && w.level == level) {
        uint32_t c[3];
        float fd[3];
        point_cell(level, x, y, z, c, fd);
        if (c[0] == w.cx && c[1] == w.cy && c[2] == w.cz) {
            hessian_win(T, ws, stride, fd, (float)(1.0 / dl), H);
            done = true;
        }
    }
    if (!done) {
        const double h = 0.5 * dl;
        const Field7 xm = tsc<false>(T, x - h, y, z, false), xp = tsc<false>(T, x + h, y, z, false);
        const Field7 ym = tsc<false>(T, x, y - h, z, false), yp = tsc<false>(T, x, y + h, z, false);
        const Field7 zm = tsc<false>(T, x, y, z - h, false), zp = tsc<false>(T, x, y, z + h, false);
        const float idl = (float)(1.0 / dl);
        H[0] = (xp.dx - xm.dx) * idl; H[1] = (yp.dx - ym.dx) * idl; H[2] = (zp.dx - zm.dx) * idl;
        H[3] = (yp.dy - ym.dy) * idl; H[4] = (zp.dy - zm.dy) * idl; H[5] = (zp.dz - zm.dz) * idl;
    }
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    const float rho = sqrtf(fx * fx + fy * fy);
    const float r = sqrtf(fx * fx + fy * fy + fz * fz);
    const float cp = (rho > 0.f) ? fx / rho : 1.f, sp = (rho > 0.f) ? fy / rho : 0.f;
    const float ct = fz / r, st = rho / r;
    const float s2p = 2.f * sp * cp, s2t = 2.f * st * ct;
    const float dxx = H[0], dxy = H[1], dxz = H[2], dyy = H[3], dyz = H[4], dzz = H[5];
    out3[0] = sp * sp * dxx + cp * cp * dyy - s2p * dxy;
    out3[1] = ct * cp * sp * (dyy - dxx) + (cp * cp - sp * sp) * ct * dxy + sp * st * dxz - cp * st * dyz;
    out3[2] = cp * cp * ct * ct * dxx + sp * sp * ct * ct * dyy + st * st * dzz + s2p * ct * ct * dxy - sp * s2t * dyz - cp * s2t * dxz;
}

// deepest cell of a point: through the window when possible
__device__ __forceinline__ Found locate_fast(const DevTree& T, const Win& w, const int* ws, int stride, double x, double y,
                                             double z)
{
    if (w.level >= 0) {
        uint32_t c[3];
        float fd[3];
        point_cell(w.level, x, y, z, c, fd);
        const int ox = (int)(c[0] - w.cx), oy = (int)(c[1] - w.cy), oz = (int)(c[2] - w.cz);
        if (abs(ox) <= 2 && abs(oy) <= 2 && abs(oz) <= 2) {
            const int e = ws[widx(ox, oy, oz) * stride];
            if (e >= 0 && !(e & kHasChildren)) return Found{e & kCellMask, w.level};
        }
    }
    return locate(T, x, y, z);
}

// CIC through the window: the 8 cells of the centre's level around the point
// (simplehyperoctree.h:1410-1469 without a restart).
__device__ __forceinline__ bool cic_win(const DevTree& T, const Win& w, const int* ws, int stride, double x, double y, double z,
                                        bool need_all, Field7& res)
{
    if (w.level < 0) return false;
    uint32_t c[3];
    float fd[3];
    point_cell(w.level, x, y, z, c, fd);
    const int ox = (int)(c[0] - w.cx), oy = (int)(c[1] - w.cy), oz = (int)(c[2] - w.cz);
    if (abs(ox) > 1 || abs(oy) > 1 || abs(oz) > 1) return false;
    const int ec = ws[widx(ox, oy, oz) * stride];
    if (ec < 0 || (ec & kHasChildren)) return false;
    // neighbour on the point's side along each axis, weights (1-|fd|, |fd|)
    const int sx = (fd[0] >= 0.f) ? 1 : -1, sy = (fd[1] >= 0.f) ? 1 : -1, sz = (fd[2] >= 0.f) ? 1 : -1;
    const float ax = fabsf(fd[0]), ay = fabsf(fd[1]), az = fabsf(fd[2]);
    int cell[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) {
        const int e = ws[widx(ox + ((v & 1) ? sx : 0), oy + ((v & 2) ? sy : 0), oz + ((v & 4) ? sz : 0)) * stride];
        if (e < 0) return false;
        cell[v] = e & kCellMask;
    }
    float gx = 0.f, gy = 0.f, gz = 0.f, gt = 0.f, rho = 0.f, phi = 0.f, a = 0.f;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
        const float wt = ((v & 1) ? ax : 1.f - ax) * ((v & 2) ? ay : 1.f - ay) * ((v & 4) ? az : 1.f - az);
        const float4 g = __ldg(T.grad + cell[v]);
        gx = fmaf(g.x, wt, gx); gy = fmaf(g.y, wt, gy); gz = fmaf(g.z, wt, gz); gt = fmaf(g.w, wt, gt);
        if (need_all) {
            const float4 s = __ldg(T.scal + cell[v]);
            rho = fmaf(s.x, wt, rho); phi = fmaf(s.y, wt, phi); a = fmaf(s.z, wt, a);
        }
    }
    res = Field7{rho, phi, gx, gy, gz, a, gt};
    return true;
}

__device__ __forceinline__ Field7 gather_fast(const DevTree& T, const Win& w, const int* ws, int stride, int order, double x,
                                              double y, double z, bool need_all)
{
    Field7 r;
    if (order == 1) {
        if (cic_win(T, w, ws, stride, x, y, z, need_all, r)) return r;
        return cic<false>(T, x, y, z, need_all);
    }
    if (tsc_win(T, w, ws, stride, x, y, z, need_all, r)) return r;
    return tsc<false>(T, x, y, z, need_all);
}

struct FastRec {
    double a, t, x, y, z, k0, k1, k2, k3;
    double phi, red, chi, lambda, s, isw, iswold;
    float rho, dx, dy, dz, dt, ah;   // dt: the photon's (forward) dphidt
    int level;
};

__device__ __forceinline__ void rhs_fast(const DevTree& T, const DevCosmo& C, const PropParams& P, const Win& w, const int* ws,
                                         int stride, double inv_scale, const double* in, double* out)
{
    const double c2 = kC * kC;
    const Field7 d = gather_fast(T, w, ws, stride, P.order, in[2], in[3], in[4], false);
    const double dphidl = (double)d.dt * in[5] + ((double)d.dx * in[6] + (double)d.dy * in[7] + (double)d.dz * in[8]);
    const double dadt = interp_fast(C, in[1], C.dadt, C.slope_dadt);
    out[0] = in[5] * dadt;
    out[1] = in[5];
    out[2] = in[6] * inv_scale;
    out[3] = in[7] * inv_scale;
    out[4] = in[8] * inv_scale;
    const double hub = 2.0 * dadt / in[0] * in[5];
    const double g = (2.0 / c2) * dphidl;
    const double k02 = 2.0 * in[5] * in[5];
    out[5] = -(hub * in[5]) - ((2.0 / c2) * in[5]) * (dphidl - (double)d.dt * in[5]);
    out[6] = -(hub * in[6]) + (g * in[6]) - ((double)d.dx * k02);
    out[7] = -(hub * in[7]) + (g * in[7]) - ((double)d.dy * k02);
    out[8] = -(hub * in[8]) + (g * in[8]) - ((double)d.dz * k02);
}

__device__ void propagate_fast(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* L, long long i,
                               const PropOut& O, int* ws, int stride)
{
    const double c2 = kC * kC;
    const double mn = -(double)kExtent / 2.0, mx = (double)kExtent / 2.0;
    const double scale = P.length;
    const double inv_scale = 1.0 / scale;
    const int np = P.nplanes;
    Win w;
    w.level = -1;
    FastRec b;
    {
        const double norm = sqrt((L[3] - L[0]) * (L[3] - L[0]) + (L[4] - L[1]) * (L[4] - L[1]) + (L[5] - L[2]) * (L[5] - L[2]));
        b.a = 1.0; b.t = 0.0; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = 1.0;
        b.k1 = (L[3] - L[0]) / norm; b.k2 = (L[4] - L[1]) / norm; b.k3 = (L[5] - L[2]) / norm;
    }
    Field7 data = gather<false>(T, P.order, b.x, b.y, b.z, true);
    {
        const double ph = (double)data.phi / c2;
        const double norm = sqrt((c2 * (1.0 + 2.0 * ph) * b.k0 * b.k0) / ((1.0 - 2.0 * ph) * (b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3)));
        b.k1 *= norm; b.k2 *= norm; b.k3 *= norm;
    }
    b.a = interp_fast(C, b.t, C.a, C.slope_a);
    Found loc = locate(T, b.x, b.y, b.z);
    b.level = (loc.cell >= 0) ? loc.level : 0;
    if (loc.cell >= 0) {
        uint32_t c[3];
        float fd[3];
        point_cell(loc.level, b.x, b.y, b.z, c, fd);
        win_build(T, loc.level, c[0], c[1], c[2], ws, stride, w);
    }
    b.ah = 0.f;
    b.rho = data.rho; b.phi = data.phi; b.dx = data.dx; b.dy = data.dy; b.dz = data.dz; b.dt = data.dt;
    b.red = 0.0; b.isw = 0.0; b.chi = 0.0; b.iswold = 0.0; b.lambda = 0.0; b.s = 0.0;
    double ratio = b.a * b.a * (scale / kC) / P.nsteps;
    double dl = (loc.cell >= 0 ? cell_extent(loc.level) : 0.0) * ratio;
    const double a0 = b.a;
    const double phi0c2 = b.phi / c2;
    float last_data_dt = data.dt;
    double last_lap = 0.0;

    int next_plane = 0;
    long long cross_k[kMaxPlanes];
    for (int j = 0; j < np; ++j) cross_k[j] = -1;
    double* prow = O.plane_rec ? O.plane_rec + (long long)i * np * kPlaneFields : nullptr;
    while (next_plane < np && ((P.stop_kind == STOP_A) ? (b.a < P.planes[next_plane])
                                                        : (((P.stop_kind == STOP_R) ? b.chi : (P.stop_kind == STOP_LAMBDA) ? b.lambda
                                                            : (P.stop_kind == STOP_T) ? b.t : (P.stop_kind == STOP_S) ? b.s : b.red) >
                                                           P.planes[next_plane]))) {
        cross_k[next_plane] = 0;
        ++next_plane;
    }
    double rmax = 0.0;
    bool have_rmax = false;
    double S[6] = {0, 0, 0, 0, 0, 0}, c_k[6] = {0, 0, 0, 0, 0, 0}, c_km1[6] = {0, 0, 0, 0, 0, 0};
    double chim1 = 0.0, chim2 = 0.0;
    long long k = 0;
    unsigned status = 0;
    double isw = 0.0, iswold = 0.0, lambda = 0.0, sacc = 0.0;
    double core[9], dc[9], acc[9];
    FastRec p;
    while (!is_empty(data)) {
        if (k >= P.max_steps) { status |= 1u; break; }
        const double bc[9] = {b.a, b.t, b.x, b.y, b.z, b.k0, b.k1, b.k2, b.k3};
        const double hdl = 0.5 * dl;
        // stage derivatives folded into acc = d0 + 2 d1 + 2 d2 + d3 in that order
        rhs_fast(T, C, P, w, ws, stride, inv_scale, bc, dc);
#pragma unroll
        for (int q = 0; q < 9; ++q) { acc[q] = dc[q]; core[q] = bc[q] + hdl * dc[q]; }
        rhs_fast(T, C, P, w, ws, stride, inv_scale, core, dc);
#pragma unroll
        for (int q = 0; q < 9; ++q) { acc[q] += 2.0 * dc[q]; core[q] = bc[q] + hdl * dc[q]; }
        rhs_fast(T, C, P, w, ws, stride, inv_scale, core, dc);
#pragma unroll
        for (int q = 0; q < 9; ++q) { acc[q] += 2.0 * dc[q]; core[q] = bc[q] + dl * dc[q]; }
        rhs_fast(T, C, P, w, ws, stride, inv_scale, core, dc);
        const double dl6 = dl * (1.0 / 6.0);
#pragma unroll
        for (int q = 0; q < 9; ++q) core[q] = bc[q] + dl6 * (acc[q] + dc[q]);
        p.a = core[0]; p.t = core[1]; p.x = core[2]; p.y = core[3]; p.z = core[4];
        p.k0 = core[5]; p.k1 = core[6]; p.k2 = core[7]; p.k3 = core[8];
        data = gather_fast(T, w, ws, stride, P.order, p.x, p.y, p.z, true);
        if (!(!(p.a < 0.0) && ((p.x > mn) && (p.x < mx) && (p.y > mn) && (p.y < mx) && (p.z > mn) && (p.z < mx)))) clear(data);
        loc = locate_fast(T, w, ws, stride, p.x, p.y, p.z);
        p.level = (loc.cell >= 0) ? loc.level : 0;
        p.ah = data.a;
        p.rho = data.rho; p.phi = data.phi; p.dx = data.dx; p.dy = data.dy; p.dz = data.dz;
        p.dt = -data.dt;
        const double lap = ((double)data.phi - b.phi) / dl;
        isw += ((double)b.dt + (double)p.dt) * (p.t - b.t) * (1.0 / c2);
        iswold -= 2.0 * (p.phi - b.phi) * (1.0 / c2) -
                  (((double)b.dx + (double)p.dx) * (p.x - b.x) * scale + ((double)b.dy + (double)p.dy) * (p.y - b.y) * scale +
                   ((double)b.dz + (double)p.dz) * (p.z - b.z) * scale) * (1.0 / c2);
        p.chi = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        lambda += dl;
        sacc += sqrt((p.x - b.x) * (p.x - b.x) + (p.y - b.y) * (p.y - b.y) + (p.z - b.z) * (p.z - b.z));
        p.red = a0 / p.a * (1.0 + phi0c2 - p.phi / c2) - 1.0;
        p.isw = isw; p.iswold = iswold; p.lambda = lambda; p.s = sacc;
        if (!is_empty(data)) {
            ratio = p.a * p.a * (scale / kC) / P.nsteps;
            dl = (loc.cell >= 0 ? cell_extent(loc.level) : 0.0) * ratio;
            last_data_dt = data.dt;
            last_lap = lap;
            // keep the window centred on the new point's cell
            if (loc.cell >= 0) {
                uint32_t c[3];
                float fd[3];
                point_cell(loc.level, p.x, p.y, p.z, c, fd);
                if (w.level != loc.level || c[0] != w.cx || c[1] != w.cy || c[2] != w.cz)
                    win_build(T, loc.level, c[0], c[1], c[2], ws, stride, w);
            }
            ++k;
            if (P.jacobian) {
                float h3[3];
                jac_fast(T, w, ws, stride, p.x, p.y, p.z, p.level, h3);
                const double dr = p.chi - b.chi;
                chim2 = chim1; chim1 = b.chi;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    c_km1[q] = c_k[q]; c_km1[3 + q] = c_k[3 + q];
                    const double hd = (double)h3[q] * dr;
                    c_k[q] = p.chi * hd;
                    c_k[3 + q] = p.chi * p.chi * hd;
                    S[q] += c_k[q];
                    S[3 + q] += c_k[3 + q];
                }
            }
            while (next_plane < np) {
                const int kind = P.stop_kind;
                const double q1 = (kind == STOP_R) ? p.chi : (kind == STOP_LAMBDA) ? p.lambda : (kind == STOP_T) ? p.t
                                : (kind == STOP_A) ? p.a : (kind == STOP_S) ? p.s : p.red;
                const double ref = P.planes[next_plane];
                if (!((kind == STOP_A) ? (q1 < ref) : (q1 > ref))) break;
                const int j = next_plane++;
                cross_k[j] = k;
                if (prow) {
                    double* o = prow + j * kPlaneFields;
                    const double q0 = (kind == STOP_R) ? b.chi : (kind == STOP_LAMBDA) ? b.lambda : (kind == STOP_T) ? b.t
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
                    if (P.jacobian) {
                        double s1[3], s2[3];
                        bool ok = true;
                        if (p.chi <= dist) {
                            for (int q = 0; q < 3; ++q) { s1[q] = S[q]; s2[q] = S[3 + q]; }
                        } else if (chim1 <= dist) {
                            for (int q = 0; q < 3; ++q) { s1[q] = S[q] - c_k[q]; s2[q] = S[3 + q] - c_k[3 + q]; }
                        } else if (k >= 2 && chim2 <= dist) {
                            for (int q = 0; q < 3; ++q) {
                                s1[q] = S[q] - c_k[q] - c_km1[q];
                                s2[q] = S[3 + q] - c_k[3 + q] - c_km1[3 + q];
                            }
                        } else {
                            ok = false;
                            status |= 2u;
                        }
                        if (ok) {
                            const double idist = 1.0 / dist;
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
        }
        bool stop;
        switch (P.stop_kind) {
        case STOP_R: stop = b.chi > P.stop_ref; break;
        case STOP_LAMBDA: stop = b.lambda > P.stop_ref; break;
        case STOP_REDSHIFT: stop = b.red > P.stop_ref; break;
        case STOP_T: stop = b.t > P.stop_ref; break;
        case STOP_A: stop = b.a < P.stop_ref; break;
        case STOP_PLANE: stop = (p.x * P.ki[0] + p.y * P.ki[1] + p.z * P.ki[2]) > P.stop_ref; break;
        case STOP_S: stop = b.s > P.stop_ref; break;
        default: stop = true;
        }
        if (stop) break;
    }
    long long size = k + 1;
    if (signbit(b.red) || signbit(b.a)) size -= 1;
    O.steps[i] = size;
    if (O.final_rec) {
        double* o = O.final_rec + i * kPhotonFields;
        if (size == k + 1) {
            Rec r;
            r.a = b.a; r.t = b.t; r.x = b.x; r.y = b.y; r.z = b.z; r.k0 = b.k0; r.k1 = b.k1; r.k2 = b.k2; r.k3 = b.k3;
            r.level = b.level; r.ah = b.ah; r.rho = b.rho; r.phi = b.phi;
            r.dx = b.dx; r.dy = b.dy; r.dz = b.dz; r.dt = b.dt;
            r.dphidl = (k > 0) ? ((double)last_data_dt * b.k0 + ((double)b.dx * b.k1 + (double)b.dy * b.k2 + (double)b.dz * b.k3)) : 0.0;
            r.lap = (k > 0) ? last_lap : 0.0;
            const double kk = b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3;
            r.ds2 = (b.a * b.a) * (-(c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0) + ((1.0 - 2.0 * (b.phi / c2)) * kk));
            r.err = 1.0 - ((1.0 - 2.0 * (b.phi / c2)) * kk) / (c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0);
            r.red = b.red; r.isw = b.isw; r.iswold = b.iswold; r.chi = b.chi; r.lambda = b.lambda; r.s = b.s;
            r.index = (double)k;
            write_rec(o, r);
        } else {
            for (int q = 0; q < kPhotonFields; ++q) o[q] = 0.0;
            status |= 4u;
        }
    }
    if (prow) {
        for (int j = 0; j < np; ++j) {
            double* o = prow + j * kPlaneFields;
            const long long ck = cross_k[j];
            const bool found = (ck >= 1) && (ck < size);
            const bool valid = found && !((ck - 1) == size - 1 || (ck - 1) == 0);
            if (ck < 0 || ck == 0 || ck >= size) {
                for (int q = 0; q < kPlaneFields; ++q) o[q] = 0.0;
                o[0] = (ck == 0) ? 0.0 : (double)(size - 1);
            }
            o[19] = valid ? 1.0 : 0.0;
        }
    }
    if (status) atomicOr(O.status, status);
}

constexpr int kFastThreads = 128;

// Persistent launch: each warp takes the next 32 rays from a global counter
// until the batch is exhausted, so uneven path lengths do not leave tail
// waves.  `queue` is zeroed before the launch.
__global__ void __launch_bounds__(kFastThreads) k_propagate_fast(DevTree T, DevCosmo C, PropParams P,
                                                                 const double* __restrict__ launch, long long n, PropOut O,
                                                                 unsigned long long* queue)
{
    extern __shared__ int smem_win[];
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(queue, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned long long)n) break;
        const long long i = (long long)base + lane;
        if (i < n) propagate_fast(T, C, P, launch + 6 * i, i, O, smem_win + threadIdx.x, blockDim.x);
        __syncwarp();
    }
}

}  // namespace mpf
