// Per-source device state and arithmetic of the catalogue root-finder,
// shared by the round-based driver (mpf_catalogue.cu, built with -fmad=false:
// the reference's operation order) and the persistent work-queue driver
// (mpf_cat_persist.cu).
#pragma once
#include "mpf_catalogue.h"

namespace mpf {

// per-source device state
struct CatState {
    double tx, ty, tz;       // source position in the octree frame
    double vx, vy, vz;       // source velocity in the octree frame
    double dist;             // |x_s|
    double phi, theta;       // current launch angles
    // bundle Jacobian (jacobiantype = bundle): the last ray's end point and
    // miss, the screen normal and the bundle's stop value (catalogues.h:458-495)
    double fx, fy, fz, miss;
    double kx, ky, kz, iref;
    int it;                  // rays traced so far (the persistent driver's per-source Newton round)
};

// Newton step in the screen basis (catalogues.h:625-655) with the inverse
// Jacobian ji; returns the new launch angles.
__device__ __forceinline__ void newton_step(const CatState& S, double fx, double fy, double fz, double ji00, double ji01,
                                            double ji10, double ji11, double& nphi, double& ntheta)
{
    const double cp = cos(S.phi), sp = sin(S.phi), ct = cos(S.theta), st = sin(S.theta);
    const double e10 = -sp, e11 = cp;
    const double e20 = -cp * ct, e21 = -sp * ct, e22 = st;
    const double g0 = S.dist * cp * st, g1 = S.dist * sp * st, g2 = S.dist * ct;
    const double sep0 = fx - S.tx, sep1 = fy - S.ty, sep2 = fz - S.tz;
    const double pos0 = g0 - S.tx, pos1 = g1 - S.ty, pos2 = g2 - S.tz;
    const double sepx = sep0 * e10 + sep1 * e11;
    const double sepy = sep0 * e20 + sep1 * e21 + sep2 * e22;
    const double posx = pos0 * e10 + pos1 * e11;
    const double posy = pos0 * e20 + pos1 * e21 + pos2 * e22;
    const double sepxnew = ji00 * sepx + ji01 * sepy;
    const double sepynew = ji10 * sepx + ji11 * sepy;
    const double posxnew = posx - sepxnew;
    const double posynew = posy - sepynew;
    const double xnew = S.tx + (posxnew * e10 + posynew * e20);
    const double ynew = S.ty + (posxnew * e11 + posynew * e21);
    const double znew = S.tz + posynew * e22;
    nphi = atan2(ynew, xnew);
    ntheta = acos(znew / sqrt(xnew * xnew + ynew * ynew + znew * znew));
}

// 2-D Morton key of a direction: 16 bits of phi in [-pi, pi] and of theta in [0, pi], interleaved.
__device__ __forceinline__ uint32_t spread16(uint32_t v)
{
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
__device__ __forceinline__ uint32_t direction_key(double phi, double theta)
{
    const double pi = 3.14159265358979323846;
    const double u = fmin(fmax((phi + pi) * (1.0 / (2.0 * pi)), 0.0), 1.0);
    const double v = fmin(fmax(theta * (1.0 / pi), 0.0), 1.0);
    return spread16((uint32_t)(u * 65535.0)) | (spread16((uint32_t)(v * 65535.0)) << 1);
}

// relCat's per-source setup (catalogues.h:818-836) for source i: its state
// (position and velocity in the octree frame, distance, the comoving first
// guess of the launch angles), its row's first columns, and its sort key:
// farthest sources first in 1/8-octave radius bins, then by direction, so
// that the 32 rays of a warp are neighbours of about the same length.
__device__ __forceinline__ void cat_init_one(long long i, const double* __restrict__ src, int stride,
                                             const CatRotation& rot, int has_rot, CatState* __restrict__ state,
                                             double* __restrict__ rows, uint32_t* __restrict__ key,
                                             int* __restrict__ val, unsigned* __restrict__ count)
{
    const double* s = src + (long long)stride * i;
    CatState S;
    double t[3], v[3];
    for (int j = 0; j < 3; ++j) {
        if (!has_rot) {
            t[j] = s[j];
            v[j] = s[j + 3];
        } else {
            // relCat (catalogues.h:818-826)
            t[j] = s[0] * rot.m[j][0] + s[1] * rot.m[j][1] + s[2] * rot.m[j][2];
            v[j] = s[3] * rot.m[j][0] + s[4] * rot.m[j][1] + s[5] * rot.m[j][2];
        }
    }
    S.tx = t[0]; S.ty = t[1]; S.tz = t[2];
    S.vx = v[0]; S.vy = v[1]; S.vz = v[2];
    S.dist = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    // comoving first guess (catalogues.h:832-836)
    S.theta = acos(t[2] / S.dist);
    S.phi = atan2(t[1], t[0]);
    S.fx = S.fy = S.fz = S.miss = 0.0;
    S.kx = S.ky = S.kz = S.iref = 0.0;
    S.it = 0;
    state[i] = S;
    double* r = rows + (long long)kCatalogueFields * i;
    for (int k = 0; k < kCatalogueFields; ++k) r[k] = 0.0;
    r[0] = S.phi;
    r[1] = S.theta;
    val[i] = (int)i;
    if (S.dist > 0.0 && isfinite(S.dist) && isfinite(S.phi) && isfinite(S.theta)) {
        // farthest sources first, in 1/8-octave radius bins (the float's
        // exponent and 3 mantissa bits), then by direction: a warp's rays have
        // about the same length, and the persistent queue starts the long ones
        // first; below the key of the excluded sources
        const uint32_t rbin = __float_as_uint((float)S.dist) >> 20;
        key[i] = ((0x7ffu - min(rbin, 0x7ffu)) << 20) | (direction_key(S.phi, S.theta) >> 12);
        atomicAdd(count, 1u);
    } else {
        key[i] = 0xffffffffu;
        // a source at the observer (or with non-finite coordinates) has no
        // direction: reported as unreachable
        r[2] = 42.0; r[3] = 42.0;
    }
}

// Outcome of one ray of a source (cat_update).
enum { kCatDone = 0, kCatContinue = 1, kCatPendBundle = 2, kCatRetrace = 3 };

// One newtonMethod2d call (catalogues.h:410-727) for source s after its ray
// came back: o = the ray's source-mode record, steps = its trajectory size.
// Writes the source's row where the reference writes its result, redshifts
// and jacobian; returns whether the source is finished (kCatDone), takes
// another ray (kCatContinue: its new angles are in state[s]), waits for a
// bundle Jacobian (kCatPendBundle) or converged and needs its Jacobian from a
// re-trace (kCatRetrace).  photon_steps[0] / [1]: all accepted steps / those
// traced with the Jacobian.
__device__ __forceinline__ int cat_update(int s, int iteration, int traced_jacobian, const CatConst& K,
                                          CatState* __restrict__ state, double* __restrict__ rows, long long steps,
                                          const double* __restrict__ o, unsigned long long* __restrict__ photon_steps)
{
    const double c = kC, c2 = kC * kC;
    CatState S = state[s];
    double* row = rows + (long long)kCatalogueFields * s;
    // photon_steps[0]: all accepted steps; [1]: those traced with the Jacobian
    const unsigned long long ns = (unsigned long long)(steps > 0 ? steps - 1 : 0);
    atomicAdd(photon_steps, ns);
    if (traced_jacobian) atomicAdd(photon_steps + 1, ns);
    const unsigned count = (unsigned)iteration + 1u;
    if (o[19] == 0.0) {
        // the ray did not reach the source radius (catalogues.h:436-442)
        row[2] = 42.0; row[3] = 42.0; row[4] = 0.0; row[5] = o[0];
        return kCatDone;
    }
    const double fx = o[2], fy = o[3], fz = o[4];
    const double scale_factor = o[10];
    row[7] = o[11];   // redshifts[1], FLRW + potential (catalogues.h:451)
    // the reference squares with pow(x, 2); x * x is the correctly rounded square
    const double ex = S.tx - fx, ey = S.ty - fy, ez = S.tz - fz;
    const double dist_sep = sqrt(ex * ex + ey * ey + ez * ez);
    const double miss = dist_sep / S.dist;
    if (K.bundle) {
        // the bundle's screen normal and stop value at this ray's end (catalogues.h:458-495)
        if (K.plane_sachs) { S.kx = o[21]; S.ky = o[22]; S.kz = o[23]; }
        else { S.kx = fx; S.ky = fy; S.kz = fz; }
        switch (K.stop_bundle) {
        case STOP_REDSHIFT: S.iref = o[11]; break;
        case STOP_A: S.iref = scale_factor; break;
        case STOP_T: S.iref = o[9]; break;
        case STOP_LAMBDA: S.iref = o[13]; break;
        case STOP_PLANE: S.iref = S.kx * fx + S.ky * fy + S.kz * fz; break;
        default: S.iref = S.dist; break;   // "r"
        }
        S.fx = fx; S.fy = fy; S.fz = fz; S.miss = miss;
        state[s] = S;
    }
    if (miss > K.accuracy && K.bundle && iteration >= 5) {
        return kCatPendBundle;   // the Newton step needs the four-ray Jacobian first
    }
    if (miss > K.accuracy) {
        double ji00 = 1.0, ji01 = 0.0, ji10 = 0.0, ji11 = 1.0;
        if (iteration >= 3) {
            // infinitesimal Jacobian at the radius; Utility::invMatrix2d (utility.h:686-696)
            const double a00 = o[6], a01 = o[7], a10 = o[7], a11 = o[8];
            row[12] = a00; row[13] = a01; row[14] = a10; row[15] = a11;
            const double invdet = 1. / (a00 * a11 - a01 * a10);
            ji00 = a11 * invdet;
            ji01 = -a01 * invdet;
            ji10 = -a10 * invdet;
            ji11 = a00 * invdet;
        }
        double nphi, ntheta;
        newton_step(S, fx, fy, fz, ji00, ji01, ji10, ji11, nphi, ntheta);
        row[2] = nphi; row[3] = ntheta; row[4] = miss;
        if (count > (unsigned)K.max_iterations) {
            row[5] = 42.0;   // rejected
            return kCatDone;
        }
        S.phi = nphi;
        S.theta = ntheta;
        state[s] = S;
        return kCatContinue;
    }
    // converged (catalogues.h:658-726)
    row[2] = S.phi; row[3] = S.theta; row[4] = miss; row[5] = (double)count;
    int outcome = kCatDone;
    if (K.bundle || K.born) {
        outcome = kCatRetrace;   // its Jacobian comes from the four-ray bundle or the Born ray after the last round
    } else if (traced_jacobian) {
        row[12] = o[6]; row[13] = o[7]; row[14] = o[7]; row[15] = o[8];
    } else {
        outcome = kCatRetrace;
    }
    const double potential = o[17];
    const double isw = o[15];
    const double z1 = o[11];
    const double z0 = -1 + 1. / (scale_factor);
    const double unit_t = scale_factor * scale_factor * K.mpc / (K.h * 100.0 * 1000.0);
    const double unit_l = scale_factor * K.length * 100;
    const double velocityx = S.vx * unit_l * 1e-2 / (unit_t * c);
    const double velocityy = S.vy * unit_l * 1e-2 / (unit_t * c);
    const double velocityz = S.vz * unit_l * 1e-2 / (unit_t * c);
    const double a0 = o[24], phi0 = o[25], k01 = o[26], k02 = o[27], k03 = o[28];
    const double dtdl0 = 1.0;   // the launch sets dtdl = 1; the normalisation scales dx/dl only
    const double* vo = K.vobs;
    const double gref = -a0 * c * dtdl0 * (1. + phi0 / c2 + (vo[0] * k01 + vo[1] * k02 + vo[2] * k03) / (c * dtdl0) +
                                           0.5 * (vo[0] * vo[0] + vo[1] * vo[1] + vo[2] * vo[2]));
    const double dtdl = o[20], dxdl = o[21], dydl = o[22], dzdl = o[23];
    const double gK = -scale_factor * c * dtdl * (1. + potential / c2 + (velocityx * dxdl + velocityy * dydl + velocityz * dzdl) / (c * dtdl) +
                                                   0.5 * (velocityx * velocityx + velocityy * velocityy + velocityz * velocityz));
    const double z2 = z1 + (velocityx * dxdl + velocityy * dydl + velocityz * dzdl) / (scale_factor * c * dtdl) -
                      (vo[0] * k01 + vo[1] * k02 + vo[2] * k03) / (scale_factor * c * dtdl0);
    const double z3 = z2 + 0.5 * (velocityx * velocityx + velocityy * velocityy + velocityz * velocityz - vo[0] * vo[0] -
                                  vo[1] * vo[1] - vo[2] * vo[2]) / scale_factor;
    const double z4 = z3 + isw / scale_factor;
    const double z5 = gK / gref - 1;
    row[6] = z0; row[7] = z1; row[8] = z2; row[9] = z3; row[10] = z4; row[11] = z5;
    return outcome;
}

// Jacobian of a converged source from its re-traced ray's record (or, for
// jacobiantype = infinitesimal_born, from its Born ray's record).
__device__ __forceinline__ void cat_final_jacobian(double* __restrict__ row, const double* __restrict__ o, long long steps,
                                                   unsigned long long* __restrict__ photon_steps, int born)
{
    const unsigned long long ns = (unsigned long long)(steps > 0 ? steps - 1 : 0);
    atomicAdd(photon_steps, ns);
    atomicAdd(photon_steps + 1, ns);
    // a Born ray short of the radius carries the Jacobian at its last point
    if (o[19] == 0.0 && !born) return;
    row[12] = o[6]; row[13] = o[7]; row[14] = o[7]; row[15] = o[8];
}

}  // namespace mpf
