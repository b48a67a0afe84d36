// Photon propagation kernel: RK4 null-geodesic integration with CIC/TSC
// interpolation (src/integrator.h:409-445 dphotondl, :648-824 integrate with
// a stop criterion), the infinitesimal lensing Jacobian fused into the step
// (src/lensing.h:399-472) and the per-surface reduction of the map driver
// (src/hmaps.h:612-676).  One photon per thread; the FP64 state lives in
// registers; only the per-photon results leave the SM.
//
// Fusing the Jacobian: the reference sums, over trajectory points i,
//     a(d) += (d - chi_i) chi_i / d * H_i * dr_i
// after the ray is finished, for each surface distance d.  Here the two
// d-independent sums S1 = sum chi H dr and S2 = sum chi^2 H dr accumulate
// during the step, and a(d) = S1 - S2 / d is read at the crossing of each
// surface, at the last point with chi <= d (the reference's upper_bound).
// The result equals the reference's up to float64 rounding of the
// re-association.
#pragma once
#include "mpf_device.cuh"

namespace mpf {

constexpr int kMaxPlanes = 16;
constexpr int kPhotonFields = 28;
constexpr int kPlaneFields = 20;
// Source mode (catalogue root-finder): one record per ray at its own stop
// radius: the 20 surface fields, then dtdl dxdl dydl dzdl interpolated at the
// radius (20-23) and the launch point's a, phi, dxdl, dydl, dzdl (24-28).
constexpr int kSourceFields = 32;
// Wide surface records (bundle Jacobian): the 20 surface fields, dtdl dxdl
// dydl dzdl interpolated at the surface (20-23) and whether the kept
// trajectory reached the surface at all (24).
constexpr int kWideFields = 32;

enum StopKind { STOP_REDSHIFT = 0, STOP_R = 1, STOP_LAMBDA = 2, STOP_T = 3, STOP_A = 4, STOP_PLANE = 5, STOP_S = 6 };

struct DevCosmo {
    const double* t;
    const double* a;
    const double* dadt;
    int n;
    // fast-mode search accelerator: lut[k] = upper_bound(t, t0 + k / lut_scale),
    // and per-interval slopes of a and da/dt
    const int* lut;
    int nlut;
    double t0, lut_scale;
    const double* slope_a;
    const double* slope_dadt;
    // per interval k (t[k], t[k+1]): slope of da/dt and width t[k+1] - t[k], in
    // FP32 (the RK4 stages' increments of da/dt from the step's start)
    const float2* seg;
};

struct PropParams {
    double length;
    double stop_ref;
    double ki[3];
    double planes[kMaxPlanes];
    long long max_steps;
    unsigned nsteps;
    int order;
    int stop_kind;
    int nplanes;
    int jacobian;
    // source mode: per-ray stop radius; the launch record is the start point
    // and a unit direction (Integrator::launch, (phi, theta) form)
    const double* ray_stop;
    // per-ray surface values (n x nplanes; the last one is the stop value), or null
    const double* ray_planes;
    // surface records of kWideFields doubles instead of kPlaneFields
    int wide;
    // launch records give the start point and the direction itself (the
    // bundle photons of Integrator::launch(photon, count, angle, rotation),
    // whose direction is not renormalised before integrate)
    int direct;
    // Order = -1 of the reference: every gather gives the homogeneous field
    // (a = 1, the rest 0).  1: the FLRW reference ray of the rays driver,
    // integrated on a uniform octree of level hom_level (every cell is of
    // that level); 2: the Born ray of hmaps / catalogues (hmaps.h:706-712,
    // catalogues.h:670-673), on the octree itself (its levels set the steps,
    // its field the Jacobian), with the Jacobian at each surface's value (a
    // radius) and, for a surface the ray never reaches, at its last point.
    // Mode 1: exact kernel only; mode 2: both kernels (the fast kernel's
    // Born instantiations).
    int homogeneous;
    int hom_level;
    // per-ray plane normals for the stop criterion "plane" with per-ray
    // surfaces (n x nplanes x 3; the last one is the stop plane's), or null
    const double* ray_ki;
    // observer velocity (parameters v0x v0y v0z, hmaps.h:80-84), read when the
    // octree carries a velocity field (integrator.h:537-538, 707-708)
    double vobs[3];
};

struct PropOut {
    long long* steps;      // n
    double* final_rec;     // n x 28, or null
    double* plane_rec;     // n x nplanes x 20, or null
    unsigned* status;      // bit 0: a ray hit max_steps
    unsigned long long* stats;   // optional path counters (fast mode), or null
    double* traj;          // n x traj_cap x 28: every trajectory point, or null
    long long traj_cap;    // points kept per ray (status bit 3 when a ray has more)
};

// Utility::interpolate (src/utility.h:441-449)
__device__ __forceinline__ double interpolate(double x0, const double* __restrict__ x, const double* __restrict__ y, int n)
{
    int first = 0, count = n;
    while (count > 0) {
        const int step = count >> 1, it = first + step;
        if (!(x0 < __ldg(x + it))) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    int i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n > 1) {
        const double xi = __ldg(x + i), xm = __ldg(x + i - 1), yi = __ldg(y + i), ym = __ldg(y + i - 1);
        return ym + ((yi - ym) * (x0 - xm) / (xi - xm));
    }
    return (n > 0) ? __ldg(y) : 0.0;
}

// Trajectory record, named as the reference's Photon<double, 3>.
struct Rec {
    double a, t, x, y, z, k0, k1, k2, k3;
    double level, ah, rho, phi, dx, dy, dz, dt, dphidl, lap, red, ds2, err, isw, iswold, chi, lambda, s, index;
};

__device__ __forceinline__ void write_rec(double* o, const Rec& r)
{
    const double v[kPhotonFields] = {r.a, r.t, r.x, r.y, r.z, r.k0, r.k1, r.k2, r.k3, r.level, r.ah, r.rho, r.phi, r.dx,
                                     r.dy, r.dz, r.dt, r.dphidl, r.lap, r.red, r.ds2, r.err, r.isw, r.iswold, r.chi,
                                     r.lambda, r.s, r.index};
#pragma unroll
    for (int k = 0; k < kPhotonFields; ++k) o[k] = v[k];
}

constexpr double kC = 299792458.0;

// the field at a point: the octree's CIC / TSC, or the homogeneous field
template <bool EXACT>
__device__ __forceinline__ Field7 field_at(const DevTree& T, const PropParams& P, double x, double y, double z, bool need_all)
{
    if (P.homogeneous) {
        Field7 h;
        clear(h);
        h.a = 1.f;
        return h;
    }
    return gather<EXACT>(T, P.order, x, y, z, need_all);
}

// the field and the velocity at a point of a velocity-field octree (the
// homogeneous field has no velocity: integrator.h:663-664)
template <bool EXACT>
__device__ __forceinline__ Field7 field_vel_at(const DevTree& T, const PropParams& P, double x, double y, double z, float* v)
{
    if (P.homogeneous) {
        v[0] = v[1] = v[2] = 0.f;
        Field7 h;
        clear(h);
        h.a = 1.f;
        return h;
    }
    return gather_vel<EXACT>(T, P.order, x, y, z, v);
}

__device__ __forceinline__ bool vel_zero(const float* v) { return v[0] == 0.f && v[1] == 0.f && v[2] == 0.f; }

__device__ __forceinline__ Found locate_at(const DevTree& T, const PropParams& P, double x, double y, double z)
{
    if (P.homogeneous == 1) return Found{0, P.hom_level};
    return locate(T, x, y, z);
}

template <bool EXACT>
__device__ __forceinline__ void rhs(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* in, double* out)
{
    const double two = 2.0;
    const double c2 = kC * kC;
    const Field7 d = field_at<EXACT>(T, P, in[2], in[3], in[4], false);
    const double dphidl = (double)d.dt * in[5] + ((double)d.dx * in[6] + (double)d.dy * in[7] + (double)d.dz * in[8]);
    const double dadt = interpolate(in[1], C.t, C.dadt, C.n);
    const double scale = P.length;
    out[0] = in[5] * dadt;
    out[1] = in[5];
    out[2] = in[6] / scale;
    out[3] = in[7] / scale;
    out[4] = in[8] / scale;
    const double hub = two * dadt / in[0] * in[5];
    out[5] = -(hub * in[5]) - (two / c2 * in[5]) * (dphidl - (double)d.dt * in[5]);
    const double g = two / c2 * dphidl;
    out[6] = -(hub * in[6]) + (g * in[6]) - (two * (double)d.dx * in[5] * in[5]);
    out[7] = -(hub * in[7]) + (g * in[7]) - (two * (double)d.dy * in[5] * in[5]);
    out[8] = -(hub * in[8]) + (g * in[8]) - (two * (double)d.dz * in[5] * in[5]);
}

__device__ __forceinline__ double plane_q(int kind, const Rec& r, const double* ki = nullptr)
{
    if (kind == STOP_PLANE && ki) return r.x * ki[0] + r.y * ki[1] + r.z * ki[2];
    switch (kind) {
    case STOP_R: return r.chi;
    case STOP_LAMBDA: return r.lambda;
    case STOP_T: return r.t;
    case STOP_A: return r.a;
    case STOP_S: return r.s;
    default: return r.red;
    }
}

__device__ __forceinline__ bool plane_crossed(int kind, const Rec& r, double ref, const double* ki = nullptr)
{
    return (kind == STOP_A) ? (r.a < ref) : (plane_q(kind, r, ki) > ref);
}

// Jacobian running sums at one trajectory point (S1: chi H dr, S2: chi^2 H dr).
struct JSum {
    double s1[3], s2[3];
};

// a11 a12 a22 of the infinitesimal Jacobian at distance d from the sums at
// the last point with chi <= d (lensing.h:459-469)
__device__ __forceinline__ void jac_from_sums(const JSum& J, double d, double length, double* A)
{
    const double c2 = 299792458.0 * 299792458.0;
    const double a11 = J.s1[0] - J.s2[0] / d;
    const double a12 = J.s1[1] - J.s2[1] / d;
    const double a22 = J.s1[2] - J.s2[2] / d;
    A[0] = 1 - 2 * a11 / c2 * length;
    A[1] = -2 * a12 / c2 * length;
    A[2] = 1 - 2 * a22 / c2 * length;
}

template <bool EXACT>
__device__ void jac_point(const DevTree& T, const Rec& p, double dr, double* H)
{
    const double x = p.x, y = p.y, z = p.z, r = p.chi;
    double cp, sp, ct, st, s2p, s2t;
    if (EXACT) {
        const double phi = atan2(y, x);
        const double theta = acos(z / r);
        cp = cos(phi); sp = sin(phi); ct = cos(theta); st = sin(theta);
        s2p = sin(2 * phi); s2t = sin(2 * theta);
    } else {
        const double rho = sqrt(x * x + y * y);
        cp = (rho > 0.0) ? x / rho : 1.0;
        sp = (rho > 0.0) ? y / rho : 0.0;
        ct = z / r;
        st = rho / r;
        s2p = 2.0 * sp * cp;
        s2t = 2.0 * st * ct;
    }
    const double dl = ldexp(1.0, (int)(kLevelShift + 1 - (int)p.level));
    const double h = 0.5 * dl;
    const Field7 xm = tsc<EXACT>(T, x - h, y, z, false);
    const Field7 xp = tsc<EXACT>(T, x + h, y, z, false);
    const Field7 ym = tsc<EXACT>(T, x, y - h, z, false);
    const Field7 yp = tsc<EXACT>(T, x, y + h, z, false);
    const Field7 zm = tsc<EXACT>(T, x, y, z - h, false);
    const Field7 zp = tsc<EXACT>(T, x, y, z + h, false);
    const double dxxp = (double)(xp.dx - xm.dx) / dl;
    const double dxyp = (double)(yp.dx - ym.dx) / dl;
    const double dxzp = (double)(zp.dx - zm.dx) / dl;
    const double dyyp = (double)(yp.dy - ym.dy) / dl;
    const double dyzp = (double)(zp.dy - zm.dy) / dl;
    const double dzzp = (double)(zp.dz - zm.dz) / dl;
    const double d1d1p = sp * sp * dxxp + cp * cp * dyyp - s2p * dxyp;
    const double d2d2p = cp * cp * ct * ct * dxxp + sp * sp * ct * ct * dyyp + st * st * dzzp + s2p * ct * ct * dxyp -
                         sp * s2t * dyzp - cp * s2t * dxzp;
    const double d1d2p = ct * cp * sp * (dyyp - dxxp) + (cp * cp - sp * sp) * ct * dxyp + sp * st * dxzp - cp * st * dyzp;
    H[0] = d1d1p * dr;
    H[1] = d1d2p * dr;
    H[2] = d2d2p * dr;
    (void)r;
}

template <bool EXACT, bool SRC>
__device__ void propagate_one(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* L, long long i,
                              const PropOut& O)
{
    const double zero = 0.0, one = 1.0, two = 2.0, six = 6.0;
    const double c2 = kC * kC;
    const double mn = 0.0 - (double)kExtent / two, mx = 0.0 + (double)kExtent / two;
    const double scale = P.length;
    const int np = SRC ? 1 : P.nplanes;
    const int kind = SRC ? (int)STOP_R : P.stop_kind;
    const double* rpl = (!SRC && P.ray_planes) ? P.ray_planes + i * np : P.planes;   // this ray's surfaces
    const double stop_ref = SRC ? P.ray_stop[i] : (P.ray_planes ? rpl[np - 1] : P.stop_ref);
    const int rec_fields = SRC ? kSourceFields : (P.wide ? kWideFields : kPlaneFields);
    Rec b;
    if (SRC || P.direct) {
        // launch, (phi, theta) form (src/integrator.h:305-329), or a bundle
        // photon (integrator.h:346-380): direction given
        b.a = one; b.t = zero; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = one;
        b.k1 = L[3]; b.k2 = L[4]; b.k3 = L[5];
        b.index = 0.0;
    } else {
        // launch (src/integrator.h:283-309, 6-argument form)
        const double norm = sqrt((L[3] - L[0]) * (L[3] - L[0]) + (L[4] - L[1]) * (L[4] - L[1]) + (L[5] - L[2]) * (L[5] - L[2]));
        b.a = one; b.t = zero; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = one;
        b.k1 = (L[3] - L[0]) / norm; b.k2 = (L[4] - L[1]) / norm; b.k3 = (L[5] - L[2]) / norm;
        b.index = 0.0;
    }
    // Velocity-field octree (the reference built with -DVELOCITYFIELD): the
    // record's velocity slots are gathered with the other fields, count in its
    // emptiness test (data != empty compares every member), and the redshift
    // takes the ISW, Doppler and observer terms (integrator.h:765-767).
    const bool velf = T.vel != nullptr;
    float vel[3] = {0.f, 0.f, 0.f};
    Field7 data = velf ? field_vel_at<EXACT>(T, P, b.x, b.y, b.z, vel) : field_at<EXACT>(T, P, b.x, b.y, b.z, true);
    {
        const double ph = (double)data.phi / c2;
        const double norm = sqrt((c2 * (one + two * ph) * b.k0 * b.k0) / ((one - two * ph) * (b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3)));
        b.k1 *= norm; b.k2 *= norm; b.k3 *= norm;
    }
    // v0n: the observer velocity along the launch direction (integrator.h:707-708)
    const double v0n = velf ? (P.vobs[0] * b.k1 + P.vobs[1] * b.k2 + P.vobs[2] * b.k3) / (kC * b.k0) : 0.0;
    b.a = interpolate(b.t, C.t, C.a, C.n);
    Found loc = locate_at(T, P, b.x, b.y, b.z);
    b.level = (loc.cell >= 0) ? (double)loc.level : 0.0;
    b.ah = zero;
    b.rho = data.rho; b.phi = data.phi; b.dx = data.dx; b.dy = data.dy; b.dz = data.dz; b.dt = data.dt;
    b.dphidl = zero; b.lap = zero; b.red = zero;
    {
        const double kk = b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3;
        b.ds2 = (b.a * b.a) * (-(c2 * (one + two * (b.phi / c2)) * b.k0 * b.k0) + ((one - two * (b.phi / c2)) * kk));
        b.err = one - ((one - two * (b.phi / c2)) * kk) / (c2 * (one + two * (b.phi / c2)) * b.k0 * b.k0);
    }
    b.isw = zero; b.chi = zero; b.iswold = zero; b.lambda = zero; b.s = zero;
    double ratio = b.a * b.a * (scale / kC) / P.nsteps;
    double dl = (loc.cell >= 0 ? cell_extent(loc.level) : 0.0) * ratio;
    const double a0 = b.a;
    const double phi0c2 = b.phi / c2;
    double* const traj = O.traj ? O.traj + i * O.traj_cap * kPhotonFields : nullptr;
    if (traj && O.traj_cap > 0) write_rec(traj, b);

    // surfaces
    int next_plane = 0;
    long long cross_k[kMaxPlanes];
    for (int j = 0; j < np; ++j) cross_k[j] = -1;
    double* prow = O.plane_rec ? O.plane_rec + (long long)i * np * rec_fields : nullptr;
    if (SRC && prow) {
        // trajectory[0] as the redshift decomposition reads it (catalogues.h:691-693)
        prow[24] = b.a; prow[25] = b.phi; prow[26] = b.k1; prow[27] = b.k2; prow[28] = b.k3;
        prow[29] = prow[30] = prow[31] = 0.0;
    }
    // a surface crossed by the first point lies at firstid 0: invalid in the map driver
    // this ray's plane normals (stop criterion "plane" with per-ray surfaces)
    const double* rki = (!SRC && P.ray_ki) ? P.ray_ki + (long long)i * np * 3 : nullptr;
    while (next_plane < np && plane_crossed(kind, b, SRC ? stop_ref : rpl[next_plane], rki ? rki + 3 * next_plane : nullptr)) {
        cross_k[next_plane] = 0;
        ++next_plane;
    }
    double rmax_before_b = 0.0;   // max rho over the points before b (std::max_element order)
    bool have_rmax = false;
    // Jacobian sums, at the current point and the two before it
    JSum S{{0, 0, 0}, {0, 0, 0}}, Sm1 = S, Sm2 = S;
    double chim1 = 0.0, chim2 = 0.0;
    long long k = 0;   // index of b
    unsigned status = 0;

    Rec p = b;
    p.isw = zero; p.iswold = zero; p.lambda = zero; p.s = zero;
    double core[9], dc0[9], dc1[9], dc2[9], dc3[9];
    while (!(is_empty(data) && vel_zero(vel))) {
        if (k >= P.max_steps) { status |= 1u; break; }
        const double bcore[9] = {b.a, b.t, b.x, b.y, b.z, b.k0, b.k1, b.k2, b.k3};
        p.index = b.index + one;
        rhs<EXACT>(T, C, P, bcore, dc0);
#pragma unroll
        for (int q = 0; q < 9; ++q) core[q] = bcore[q] + dl / two * dc0[q];
        rhs<EXACT>(T, C, P, core, dc1);
#pragma unroll
        for (int q = 0; q < 9; ++q) core[q] = bcore[q] + dl / two * dc1[q];
        rhs<EXACT>(T, C, P, core, dc2);
#pragma unroll
        for (int q = 0; q < 9; ++q) core[q] = bcore[q] + dl * dc2[q];
        rhs<EXACT>(T, C, P, core, dc3);
#pragma unroll
        for (int q = 0; q < 9; ++q) core[q] = bcore[q] + (dl / six) * (dc0[q] + two * dc1[q] + two * dc2[q] + dc3[q]);
        p.a = core[0]; p.t = core[1]; p.x = core[2]; p.y = core[3]; p.z = core[4];
        p.k0 = core[5]; p.k1 = core[6]; p.k2 = core[7]; p.k3 = core[8];
        data = velf ? field_vel_at<EXACT>(T, P, p.x, p.y, p.z, vel) : field_at<EXACT>(T, P, p.x, p.y, p.z, true);
        if (!(!(p.a < zero) && ((p.x > mn) && (p.x < mx) && (p.y > mn) && (p.y < mx) && (p.z > mn) && (p.z < mx)))) {
            clear(data);
            vel[0] = vel[1] = vel[2] = 0.f;
        }
        loc = locate_at(T, P, p.x, p.y, p.z);
        p.level = (loc.cell >= 0) ? (double)loc.level : 0.0;
        p.ah = data.a;
        p.rho = data.rho; p.phi = data.phi; p.dx = data.dx; p.dy = data.dy; p.dz = data.dz;
        p.dt = -(double)data.dt;
        p.dphidl = (double)data.dt * p.k0 + (p.dx * p.k1 + p.dy * p.k2 + p.dz * p.k3);
        p.lap = ((double)data.phi - b.phi) / dl;
        {
            const double kk = p.k1 * p.k1 + p.k2 * p.k2 + p.k3 * p.k3;
            p.ds2 = (p.a * p.a) * ((-c2 * (one + two * (p.phi / c2)) * p.k0 * p.k0) + ((one - two * (p.phi / c2)) * kk));
            p.err = one - ((one - two * (p.phi / c2)) * kk) / (c2 * (one + two * (p.phi / c2)) * p.k0 * p.k0);
        }
        p.isw += (b.dt + p.dt) * (p.t - b.t) / c2;
        p.iswold -= 2 * (p.phi - b.phi) / c2 -
                    ((b.dx + p.dx) * (p.x - b.x) * scale + (b.dy + p.dy) * (p.y - b.y) * scale + (b.dz + p.dz) * (p.z - b.z) * scale) / c2;
        p.chi = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        p.lambda += dl;
        p.s += sqrt((p.x - b.x) * (p.x - b.x) + (p.y - b.y) * (p.y - b.y) + (p.z - b.z) * (p.z - b.z));
        if (velf) {
            const double dop = ((double)vel[0] * p.k1 + (double)vel[1] * p.k2 + (double)vel[2] * p.k3) / (kC * p.k0);
            p.red = a0 / p.a * (one + phi0c2 - p.phi / c2 + p.isw + dop - v0n) - one;
        } else {
            p.red = a0 / p.a * (one + phi0c2 - p.phi / c2) - one;
        }
        bool appended = false;
        if (!(is_empty(data) && vel_zero(vel))) {
            ratio = p.a * p.a * (scale / kC) / P.nsteps;
            dl = (loc.cell >= 0 ? cell_extent(loc.level) : 0.0) * ratio;
            appended = true;
        }
        if (appended) {
            // the new point p becomes trajectory[k+1]; b is trajectory[k]
            ++k;
            if (P.jacobian) {
                double H[3];
                jac_point<EXACT>(T, p, p.chi - b.chi, H);
                Sm2 = Sm1; Sm1 = S;
                chim2 = chim1; chim1 = b.chi;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    S.s1[q] += p.chi * H[q];
                    S.s2[q] += p.chi * p.chi * H[q];
                }
            }
            while (next_plane < np && plane_crossed(kind, p, SRC ? stop_ref : rpl[next_plane], rki ? rki + 3 * next_plane : nullptr)) {
                const int j = next_plane++;
                cross_k[j] = k;
                if (prow) {
                    double* o = prow + j * rec_fields;
                    const double ref = SRC ? stop_ref : rpl[j];
                    const double* kj = rki ? rki + 3 * j : nullptr;
                    const double q1 = plane_q(kind, p, kj), q0 = plane_q(kind, b, kj);
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
                    o[16] = b.rho * f + p.rho * (1 - f);
                    o[17] = b.phi * f + p.phi * (1 - f);
                    // max rho over points [0, firstid) = [0, k-1): all points before b
                    o[18] = have_rmax ? rmax_before_b : 0.0;
                    o[19] = 1.0;
                    if (SRC || P.wide) {
                        o[20] = b.k0 * f + p.k0 * (1 - f);
                        o[21] = b.k1 * f + p.k1 * (1 - f);
                        o[22] = b.k2 * f + p.k2 * (1 - f);
                        o[23] = b.k3 * f + p.k3 * (1 - f);
                    }
                    if (P.jacobian) {
                        // the Jacobian at the surface's distance (hmaps.h:653-656),
                        // or at the source radius or Born surface radius itself
                        // (catalogues.h:517, hmaps.h:712)
                        const double jd = (SRC || P.homogeneous == 2) ? ref : dist;
                        // last point with chi <= jd among k, k-1, k-2
                        const JSum* J = nullptr;
                        if (p.chi <= jd) J = &S;
                        else if (chim1 <= jd) J = &Sm1;
                        else if (k >= 2 && chim2 <= jd) J = &Sm2;
                        double A[3] = {1.0, 0.0, 1.0};
                        if (J) {
                            jac_from_sums(*J, jd, P.length, A);
                        } else {
                            status |= 2u;
                        }
                        o[6] = A[0]; o[7] = A[1]; o[8] = A[2];
                    } else {
                        o[6] = o[7] = o[8] = 0.0;
                    }
                }
            }
            // b moves behind the new point: fold it into the running maximum
            if (!have_rmax || rmax_before_b < b.rho) rmax_before_b = b.rho;
            have_rmax = true;
            b = p;
            if (traj) {
                if (k < O.traj_cap) write_rec(traj + k * kPhotonFields, b);
                else status |= 8u;
            }
        }
        // stop test on trajectory.back()
        bool stop = false;
        switch (kind) {
        case STOP_R: stop = b.chi > stop_ref; break;
        case STOP_LAMBDA: stop = b.lambda > stop_ref; break;
        case STOP_REDSHIFT: stop = b.red > stop_ref; break;
        case STOP_T: stop = b.t > stop_ref; break;
        case STOP_A: stop = b.a < stop_ref; break;
        case STOP_PLANE: {
            const double* kk = rki ? rki + 3 * (np - 1) : P.ki;
            stop = (p.x * kk[0] + p.y * kk[1] + p.z * kk[2]) > stop_ref;
            break;
        }
        case STOP_S: stop = b.s > stop_ref; break;
        default: stop = true;
        }
        if (stop) break;
    }
    // drop the last point when its redshift or scale factor is negative
    long long size = k + 1;
    if (signbit(b.red) || signbit(b.a)) size -= 1;
    O.steps[i] = size;
    if (O.final_rec) {
        double* o = O.final_rec + i * kPhotonFields;
        if (size == k + 1) write_rec(o, b);
        else {
            // the popped point is not reported; the record before it is not kept,
            // so report zeros with the step count (only rays ending at z<0 or a<0)
            for (int q = 0; q < kPhotonFields; ++q) o[q] = 0.0;
            status |= 4u;
        }
    }
    if (SRC && prow) {
        // the source is reached when the last kept point is the crossing
        // (catalogues.h:433-442: marked > 0 and chi(marked) >= radius)
        const long long ck = cross_k[0];
        const bool ok = (ck >= 1) && (ck < size);
        if (!ok) {
            for (int q = 0; q < 24; ++q) prow[q] = 0.0;
            const long long marked = size - 1;
            prow[0] = (double)(marked - (marked > 0));
            // a Born ray that ends short of the radius: the Jacobian at its last point
            if (P.homogeneous == 2 && P.jacobian && ck < 0) jac_from_sums(S, stop_ref, P.length, prow + 6);
        }
        prow[19] = ok ? 1.0 : 0.0;
    } else if (prow) {
        for (int j = 0; j < np; ++j) {
            double* o = prow + j * rec_fields;
            const long long ck = cross_k[j];
            const bool found = (ck >= 1) && (ck < size);
            // map driver: firstid == size-1 or firstid == 0 -> invalid
            const bool valid = found && !((ck - 1) == size - 1 || (ck - 1) == 0);
            if (ck < 0 || ck == 0 || ck >= size) {
                for (int q = 0; q < (P.wide ? 24 : kPlaneFields); ++q) o[q] = 0.0;
                o[0] = (ck == 0) ? 0.0 : (double)(size - 1);
            }
            o[19] = valid ? 1.0 : 0.0;
            if (P.wide) o[24] = found ? 1.0 : 0.0;
            if (P.homogeneous == 2) {
                // Born ray (hmaps.h:712, 719): the Jacobian at the surface radius
                // (from the last point when the ray never got there); only a
                // ray that could not take a step is unusable
                if (P.jacobian && ck < 0) jac_from_sums(S, rpl[j], P.length, o + 6);
                o[19] = (size > 1) ? 1.0 : 0.0;
            }
        }
    }
    if (status) atomicOr(O.status, status);
}

template <bool EXACT, bool SRC>
__global__ void __launch_bounds__(128) k_propagate(DevTree T, DevCosmo C, PropParams P, const double* __restrict__ launch,
                                                   long long n, PropOut O)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    propagate_one<EXACT, SRC>(T, C, P, launch + 6 * i, i, O);
}

}  // namespace mpf
