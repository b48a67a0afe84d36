// Catalogue root-finder on the device: Catalogues::iterateNewtonMethod and
// newtonMethod2d (src/catalogues.h:410-783) with jacobiantype =
// "infinitesimal" and use_previous_catalogues = 0, for a whole batch of
// sources at once.
//
// One Newton round = one batched ray launch over the still-active sources:
//   k_cat_rays    builds each active source's launch record and stop radius;
//   propagate     integrates the rays in source mode (stop at the radius, one
//                 record per ray: the crossing, the fused Jacobian at the
//                 radius, the wave-vector there and at the observer);
//   k_cat_update  measures the miss, writes the row, and either finishes the
//                 source or takes a Newton step and queues it for the next
//                 round (atomic compaction into the other active list).
// Rounds 0-2 use the identity as Newton Jacobian (catalogues.h:507-513) and
// trace without the lensing Jacobian; a source that converges there is traced
// once more with it after the last round (the ray is the same: the launch
// angles and radius are unchanged and the integration is deterministic).
//
// This unit is compiled with -fmad=false: the row arithmetic keeps the
// reference's operation order (the trigonometric functions are CUDA's).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mpf_internal.h"
#include "mpf_catalogue.h"

namespace mpf {

// per-source device state
struct CatState {
    double tx, ty, tz;       // source position in the octree frame
    double vx, vy, vz;       // source velocity in the octree frame
    double dist;             // |x_s|
    double phi, theta;       // current launch angles
    double pad;
};

__global__ void k_cat_init(long long n, const double* __restrict__ src, int stride, CatRotation rot, int has_rot,
                           CatState* __restrict__ state, double* __restrict__ rows, int* __restrict__ active,
                           unsigned* __restrict__ count)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
    S.pad = 0.0;
    state[i] = S;
    double* r = rows + (long long)kCatalogueFields * i;
    for (int k = 0; k < kCatalogueFields; ++k) r[k] = 0.0;
    r[0] = S.phi;
    r[1] = S.theta;
    if (S.dist > 0.0 && isfinite(S.dist) && isfinite(S.phi) && isfinite(S.theta)) {
        active[atomicAdd(count, 1u)] = (int)i;
    } else {
        // a source at the observer (or with non-finite coordinates) has no
        // direction: reported as unreachable
        r[2] = 42.0; r[3] = 42.0;
    }
}

// Launch records (start at the observer, unit direction of the (phi, theta)
// launch form, integrator.h:305-329) and stop radii of the active sources.
__global__ void k_cat_rays(long long m, const int* __restrict__ list, const CatState* __restrict__ state,
                           double* __restrict__ launch, double* __restrict__ radius)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const CatState& S = state[list[j]];
    double* L = launch + 6 * j;
    L[0] = 0.0; L[1] = 0.0; L[2] = 0.0;
    L[3] = cos(S.phi) * sin(S.theta);
    L[4] = sin(S.phi) * sin(S.theta);
    L[5] = cos(S.theta);
    radius[j] = S.dist;
}

// One newtonMethod2d call per active source after its ray came back, then the
// bookkeeping of iterateNewtonMethod (catalogues.h:769-780).
__global__ void k_cat_update(long long m, int iteration, int traced_jacobian, CatConst K,
                             const int* __restrict__ list, CatState* __restrict__ state, double* __restrict__ rows,
                             const long long* __restrict__ steps, const double* __restrict__ rec,
                             int* __restrict__ next, unsigned* __restrict__ next_count, int* __restrict__ retrace,
                             unsigned* __restrict__ retrace_count, unsigned long long* __restrict__ photon_steps)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const double c = kC, c2 = kC * kC;
    const int s = list[j];
    CatState S = state[s];
    double* row = rows + (long long)kCatalogueFields * s;
    const double* o = rec + (long long)kSourceFields * j;
    // photon_steps[0]: all accepted steps; [1]: those traced with the Jacobian
    const unsigned long long ns = (unsigned long long)(steps[j] > 0 ? steps[j] - 1 : 0);
    atomicAdd(photon_steps, ns);
    if (traced_jacobian) atomicAdd(photon_steps + 1, ns);
    const unsigned count = (unsigned)iteration + 1u;
    if (o[19] == 0.0) {
        // the ray did not reach the source radius (catalogues.h:436-442)
        row[2] = 42.0; row[3] = 42.0; row[4] = 0.0; row[5] = o[0];
        return;
    }
    const double fx = o[2], fy = o[3], fz = o[4];
    const double scale_factor = o[10];
    row[7] = o[11];   // redshifts[1], FLRW + potential (catalogues.h:451)
    // the reference squares with pow(x, 2); x * x is the correctly rounded square
    const double ex = S.tx - fx, ey = S.ty - fy, ez = S.tz - fz;
    const double dist_sep = sqrt(ex * ex + ey * ey + ez * ez);
    const double miss = dist_sep / S.dist;
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
        // Newton step in the screen basis (catalogues.h:625-655)
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
        const double nphi = atan2(ynew, xnew);
        const double ntheta = acos(znew / sqrt(xnew * xnew + ynew * ynew + znew * znew));
        row[2] = nphi; row[3] = ntheta; row[4] = miss;
        if (count > (unsigned)K.max_iterations) {
            row[5] = 42.0;   // rejected
            return;
        }
        S.phi = nphi;
        S.theta = ntheta;
        state[s] = S;
        next[atomicAdd(next_count, 1u)] = s;
        return;
    }
    // converged (catalogues.h:658-726)
    row[2] = S.phi; row[3] = S.theta; row[4] = miss; row[5] = (double)count;
    if (traced_jacobian) {
        row[12] = o[6]; row[13] = o[7]; row[14] = o[7]; row[15] = o[8];
    } else {
        retrace[atomicAdd(retrace_count, 1u)] = s;
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
}

// Jacobian of a converged source whose last ray was traced without it.
__global__ void k_cat_jacobian(long long m, const int* __restrict__ list, const double* __restrict__ rec,
                               const long long* __restrict__ steps, double* __restrict__ rows,
                               unsigned long long* __restrict__ photon_steps)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const unsigned long long ns = (unsigned long long)(steps[j] > 0 ? steps[j] - 1 : 0);
    atomicAdd(photon_steps, ns);
    atomicAdd(photon_steps + 1, ns);
    const double* o = rec + (long long)kSourceFields * j;
    double* row = rows + (long long)kCatalogueFields * list[j];
    if (o[19] == 0.0) return;
    row[12] = o[6]; row[13] = o[7]; row[14] = o[7]; row[15] = o[8];
}

namespace {
unsigned blocks(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

struct CatBuffers {
    void* p[10] = {};
    ~CatBuffers()
    {
        for (void* q : p)
            if (q) cudaFree(q);
    }
};
}  // namespace

cudaError_t catalogue_newton(const DevTree& T, const DevCosmo& Cs, const CatConst& K, const CatRotation* rot,
                             bool exact, int order, unsigned nsteps, long long n, const double* d_src, int stride,
                             double* d_rows, CatRunStats* stats, unsigned* h_status, cudaStream_t stream)
{
    *h_status = 0;
    stats->rays = 0;
    stats->photon_steps = 0;
    stats->photon_steps_jacobian = 0;
    stats->iterations = 0;
    stats->launches = 0;
    if (n <= 0) return cudaSuccess;
    const int tpb = 128;
    CatBuffers B;
    CatState* state = nullptr;
    int *act0 = nullptr, *act1 = nullptr, *retr = nullptr;
    unsigned* counters = nullptr;            // [0] active, [1] next, [2] retrace, [3] status
    unsigned long long* psteps = nullptr;
    double *launch = nullptr, *radius = nullptr, *rec = nullptr;
    long long* steps = nullptr;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](int k, size_t bytes) -> void* {
        if (e != cudaSuccess) return nullptr;
        e = cudaMalloc(&B.p[k], bytes);
        return (e == cudaSuccess) ? B.p[k] : nullptr;
    };
    state = (CatState*)alloc(0, (size_t)n * sizeof(CatState));
    act0 = (int*)alloc(1, (size_t)n * sizeof(int));
    act1 = (int*)alloc(2, (size_t)n * sizeof(int));
    retr = (int*)alloc(3, (size_t)n * sizeof(int));
    counters = (unsigned*)alloc(4, 8 * sizeof(unsigned));
    psteps = (unsigned long long*)alloc(5, 2 * sizeof(unsigned long long));
    launch = (double*)alloc(6, (size_t)n * 6 * sizeof(double));
    radius = (double*)alloc(7, (size_t)n * sizeof(double));
    rec = (double*)alloc(8, (size_t)n * kSourceFields * sizeof(double));
    steps = (long long*)alloc(9, (size_t)n * sizeof(long long));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(psteps, 0, 2 * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    CatRotation R{};
    if (rot) R = *rot;
    k_cat_init<<<blocks(n, tpb), tpb, 0, stream>>>(n, d_src, stride, R, rot ? 1 : 0, state, d_rows, act0, counters);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    stats->launches = 1;
    unsigned m = 0;
    if ((e = cudaMemcpyAsync(&m, counters, sizeof(unsigned), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;

    PropParams P;
    memset(&P, 0, sizeof(P));
    P.length = K.length;
    P.max_steps = 100000000ll;
    P.nsteps = nsteps;
    P.order = order;
    P.stop_kind = STOP_R;
    P.nplanes = 1;
    P.ray_stop = radius;
    PropOut O{steps, nullptr, rec, counters + 3, nullptr};
    int* cur = act0;
    int* nxt = act1;
    for (int it = 0; it <= K.max_iterations && m > 0; ++it) {
        const int jac = (it >= 3) ? 1 : 0;
        P.jacobian = jac;
        k_cat_rays<<<blocks(m, tpb), tpb, 0, stream>>>(m, cur, state, launch, radius);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = exact ? launch_propagate<true>(T, Cs, P, launch, m, O, stream) : launch_propagate<false>(T, Cs, P, launch, m, O, stream);
        if (e != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(counters + 1, 0, sizeof(unsigned), stream)) != cudaSuccess) return e;
        k_cat_update<<<blocks(m, tpb), tpb, 0, stream>>>(m, it, jac, K, cur, state, d_rows, steps, rec, nxt, counters + 1,
                                                          retr, counters + 2, psteps);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        stats->rays += m;
        stats->iterations = it + 1;
        stats->launches += 3;
        if ((e = cudaMemcpyAsync(&m, counters + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
        std::swap(cur, nxt);
    }
    // Jacobian of the sources that converged in the identity-Jacobian rounds
    unsigned r = 0;
    if ((e = cudaMemcpyAsync(&r, counters + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    if (r > 0) {
        P.jacobian = 1;
        k_cat_rays<<<blocks(r, tpb), tpb, 0, stream>>>(r, retr, state, launch, radius);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = exact ? launch_propagate<true>(T, Cs, P, launch, r, O, stream) : launch_propagate<false>(T, Cs, P, launch, r, O, stream);
        if (e != cudaSuccess) return e;
        k_cat_jacobian<<<blocks(r, tpb), tpb, 0, stream>>>(r, retr, rec, steps, d_rows, psteps);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        stats->rays += r;
        stats->launches += 3;
    }
    unsigned long long ps[2] = {0, 0};
    if ((e = cudaMemcpyAsync(ps, psteps, sizeof(ps), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_status, counters + 3, sizeof(unsigned), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    stats->photon_steps = (long long)ps[0];
    stats->photon_steps_jacobian = (long long)ps[1];
    return cudaSuccess;
}

}  // namespace mpf
