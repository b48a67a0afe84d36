// Ray bundles of the rays driver: Integrator::propagate (integrator.h:861-1015)
// for many central photons at once.
//
//  * Host: the bundle's launch directions, Integrator::launch(photon, count,
//    angle, rotation) with Center = true (integrator.h:346-380), in the
//    reference's float64 expression order (compiled without FMA contraction).
//  * Device: every ray of every bundle in one persistent launch of the
//    propagate kernel with direction launches, no stop criterion (the
//    integrate overload of integrator.h:477-618 runs until the data is empty)
//    and per-ray trajectory records.
//  * Device (k_bundle): one block per bundle; thread 0 runs the bundle checks
//    in the reference's order (a ray of size 0 ends the loop; every ray must
//    travel more than a quarter of the extent and, with a normal amin, end
//    with a data scale factor at or below it; the travelled lengths must
//    agree to 1/8), then the threads take the central ray's points: each
//    bundle ray's position is interpolated (Utility::interpolate) at the
//    central point's reference parameter, the mean separation is converted to
//    an angular diameter distance (length a / angle), and the central
//    trajectory is written in the trajectory file's column order.
// The unit is compiled with -fmad=false: the float64 arithmetic keeps the
// reference's rounding.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpf_gb300.h"
#include "mpf_internal.h"

namespace mpf {
namespace rays {

constexpr int kFileFields = 29;

// std::isnormal: finite, non-zero and not subnormal
__device__ __forceinline__ bool normal_value(double x)
{
    const double a = fabs(x);
    return a >= 2.2250738585072014e-308 && a <= 1.7976931348623157e308;
}

// the reference parameter of trajectory point k (integrator.h:925-969)
__device__ __forceinline__ double ref_param(const double* tr, long long k, int kind)
{
    const double* p = tr + k * kPhotonFields;
    switch (kind) {
    case STOP_A: return 1 / p[0] - 1;
    case STOP_T: return p[1];
    case STOP_LAMBDA: return p[25];
    case STOP_R: {
        const double dx = p[2] - tr[2], dy = p[3] - tr[3], dz = p[4] - tr[4];
        return sqrt(dx * dx + dy * dy + dz * dz);
    }
    default: return p[19];   // redshift (also for any other name)
    }
}

// Utility::interpolate(x0, ref, coordinate q) over one ray's n points (utility.h:441-449)
__device__ __forceinline__ double interp_ray(double x0, const double* tr, long long n, int kind, int q)
{
    long long first = 0, count = n;
    while (count > 0) {
        const long long step = count >> 1, it = first + step;
        if (!(x0 < ref_param(tr, it, kind))) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    long long i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n > 1) {
        const double xm = ref_param(tr, i - 1, kind), xi = ref_param(tr, i, kind);
        const double ym = tr[(i - 1) * kPhotonFields + q], yi = tr[i * kPhotonFields + q];
        return ym + ((yi - ym) * (x0 - xm) / (xi - xm));
    }
    return (n > 0) ? tr[q] : 0.0;
}

// traj: bundles x (count + 1) rays x cap points x 28; steps: the rays' sizes
__global__ void k_bundle(const double* __restrict__ traj, const long long* __restrict__ steps, long long nb, int count,
                         long long cap, int kind, double amin, double length, double angle, double* out, long long* sizes)
{
    const long long b = blockIdx.x;
    if (b >= nb) return;
    const int nt_total = count + 1;
    const double* T0 = traj + (b * nt_total) * cap * kPhotonFields;
    const long long* st = steps + b * nt_total;
    __shared__ unsigned s_nt;
    if (threadIdx.x == 0) {
        const double quarter = ((double)kExtent / (2.0 * 1.0)) / 2.0;
        const double limit = 1.0 / (2.0 * 2.0 * 2.0);
        unsigned nt = (unsigned)nt_total;
        double mx = 0.0, mn = 0.0;
        int visited = 0;
        for (unsigned it = 0; it < nt; ++it) {
            const long long size = st[it];
            double last = 0.0;
            if (!size) {
                nt = 0;
            } else {
                const double* tr = T0 + (long long)it * cap * kPhotonFields;
                const double* back = tr + (size - 1) * kPhotonFields;
                const double cx = back[2] - tr[2], cy = back[3] - tr[3], cz = back[4] - tr[4];
                last = sqrt(cx * cx + cy * cy + cz * cz);
                nt *= (last > quarter);
                const double ah = back[10];
                nt *= (!(normal_value(amin) && normal_value(ah) && (ah < 1.0))) || (!(ah > amin));
            }
            mx = (visited == 0) ? last : fmax(mx, last);
            mn = (visited == 0) ? last : fmin(mn, last);
            ++visited;
        }
        // entries never reached keep their initial zero
        if (visited < nt_total) mn = fmin(mn, 0.0);
        nt *= (fabs(mx - mn) / mx < limit);
        s_nt = nt;
    }
    __syncthreads();
    const unsigned nt = s_nt;
    const long long size0 = st[0];
    if (nt == 0) {
        if (threadIdx.x == 0) sizes[b] = 0;
        return;
    }
    if (threadIdx.x == 0) sizes[b] = size0;
    double* o_b = out + b * cap * kFileFields;
    for (long long k = threadIdx.x; k < size0; k += blockDim.x) {
        const double* p = T0 + k * kPhotonFields;
        double d = 0.0;
        if (nt > 1) {
            const double x0 = ref_param(T0, k, kind);
            for (unsigned it = 1; it < nt; ++it) {
                const double* tr = T0 + (long long)it * cap * kPhotonFields;
                const long long n = st[it];
                const double cx = interp_ray(x0, tr, n, kind, 2) - p[2];
                const double cy = interp_ray(x0, tr, n, kind, 3) - p[3];
                const double cz = interp_ray(x0, tr, n, kind, 4) - p[4];
                d += sqrt(cx * cx + cy * cy + cz * cz);
            }
            d /= (double)(nt - 1);
            d *= (length * p[0]) / angle;
        }
        double* o = o_b + k * kFileFields;
        // file order: index a t x y z dtdl dxdl dydl dzdl level ah rho phi dphidx dphidy dphidz dphidl
        // laplacian redshift dsdl2 error distance isw iswold chi lambda dphidt s
        o[0] = p[27];
        for (int q = 0; q < 9; ++q) o[1 + q] = p[q];
        o[10] = p[9]; o[11] = p[10]; o[12] = p[11]; o[13] = p[12];
        o[14] = p[13]; o[15] = p[14]; o[16] = p[15]; o[17] = p[17]; o[18] = p[18];
        o[19] = p[19]; o[20] = p[20]; o[21] = p[21]; o[22] = d;
        o[23] = p[22]; o[24] = p[23]; o[25] = p[24]; o[26] = p[25]; o[27] = p[16]; o[28] = p[26];
    }
}

// Integrator::launch(photon, count, angle, rotation) with the centre first
// (integrator.h:346-380): directions of the count + 1 photons, 3 each.
static void bundle_directions(const double* k, unsigned count, double angle, double rotation, double* dirs)
{
    const double zero = 0, one = 1, four = 4;
    const double pi = four * std::atan(one);
    const double step = (pi + pi) / double(count + (!count));
    const double r = std::sqrt((k[0] * k[0]) + (k[1] * k[1]) + (k[2] * k[2]));
    const double rcos = r * std::cos(angle);
    const double rsin = r * std::sin(angle);
    const double costheta = std::cos(std::acos(k[2] / r));
    const double sintheta = std::sin(std::acos(k[2] / r));
    const double cosphi = std::cos(std::atan2(k[1], k[0]));
    const double sinphi = std::sin(std::atan2(k[1], k[0]));
    const double cospsi = std::cos(rotation);
    const double sinpsi = std::sin(rotation);
    for (unsigned q = 0; q <= count; ++q)
        for (int d = 0; d < 3; ++d) dirs[3 * q + d] = k[d];
    if (r > zero) {
        for (unsigned istep = 0; istep < count; ++istep) {
            const double x = rsin * std::cos(istep * step);
            const double y = rsin * std::sin(istep * step);
            const double z = rcos;
            double* o = dirs + 3 * (istep + 1);
            o[0] = -cosphi * sinpsi * costheta * x - cosphi * cospsi * costheta * y + cosphi * sintheta * z + sinphi * sinpsi * y -
                   sinphi * cospsi * x;
            o[1] = -sinphi * sinpsi * costheta * x - sinphi * cospsi * costheta * y - cosphi * sinpsi * y + cosphi * cospsi * x +
                   sintheta * sinphi * z;
            o[2] = sintheta * sinpsi * x + sintheta * cospsi * y + costheta * z;
        }
    }
}

}  // namespace rays
}  // namespace mpf

using namespace mpf;

namespace {
int fail(int code, const std::string& m) { return mpf_internal_set_error(code, m.c_str()); }
int cuda_fail(cudaError_t e, const char* where)
{
    return fail(e == cudaErrorMemoryAllocation ? MPF_OUT_OF_MEMORY : MPF_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}
struct Dev {
    void* p = nullptr;
    cudaError_t alloc(size_t n) { return n ? cudaMalloc(&p, n) : cudaSuccess; }
    ~Dev()
    {
        if (p) cudaFree(p);
    }
};
}  // namespace

extern "C" int mpf_rays_propagate(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, const mpf_bundle_params* bp,
                                  int64_t n, const double* photons, const double* rotation, int64_t* sizes, double* central)
{
    if (!o || !c || !p || !bp || n < 0 || (n > 0 && (!photons || !sizes || !central)))
        return fail(MPF_BAD_INPUT, "mpf_rays_propagate: bad argument");
    if (bp->count < 0 || !(bp->angle > 0.0) || bp->capacity < 1 || p->nsteps == 0 || p->order < 0 || p->order > 2 ||
        !(p->length > 0.0) || bp->interpolation < 0 || bp->interpolation > 6 || bp->homogeneous_level > 30)
        return fail(MPF_BAD_INPUT, "mpf_rays_propagate: bad parameters");
    if (n == 0) return MPF_OK;
    const int nt = bp->count + 1;
    const long long cap = bp->capacity;
    const size_t per_bundle = (size_t)nt * cap * kPhotonFields * sizeof(double);
    const long long chunk = std::max<long long>(1, std::min<long long>(n, (long long)((size_t)2 << 30) / (long long)per_bundle));
    PropParams P;
    std::memset(&P, 0, sizeof(P));
    P.length = p->length;
    P.stop_ref = INFINITY;   // no stop criterion: integrate until the data is empty
    P.max_steps = (p->max_steps > 0) ? p->max_steps : 100000000ll;
    P.nsteps = p->nsteps;
    P.order = p->order;
    P.stop_kind = STOP_R;
    P.direct = 1;
    const bool hom = bp->homogeneous_level >= 0;
    P.homogeneous = hom ? 1 : 0;
    P.hom_level = hom ? bp->homogeneous_level : 0;
    const DevCosmo C = dev_cosmo(c);
    Dev dl, dsteps, dtraj, dout, dsizes, dstatus;
    cudaError_t e = dl.alloc((size_t)chunk * nt * 6 * sizeof(double));
    if (e == cudaSuccess) e = dsteps.alloc((size_t)chunk * nt * sizeof(long long));
    if (e == cudaSuccess) e = dtraj.alloc((size_t)chunk * per_bundle);
    if (e == cudaSuccess) e = dout.alloc((size_t)chunk * cap * rays::kFileFields * sizeof(double));
    if (e == cudaSuccess) e = dsizes.alloc((size_t)chunk * sizeof(long long));
    if (e == cudaSuccess) e = dstatus.alloc(sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "mpf_rays_propagate");
    std::vector<double> launch((size_t)chunk * nt * 6), dirs((size_t)nt * 3);
    int rc = MPF_OK;
    for (long long b0 = 0; b0 < n; b0 += chunk) {
        const long long m = std::min<long long>(chunk, n - b0);
        for (long long b = 0; b < m; ++b) {
            const double* ph = photons + (b0 + b) * 6;
            rays::bundle_directions(ph + 3, (unsigned)bp->count, bp->angle, rotation ? rotation[b0 + b] : 0.0, dirs.data());
            for (int q = 0; q < nt; ++q) {
                double* L = launch.data() + ((size_t)b * nt + q) * 6;
                L[0] = ph[0]; L[1] = ph[1]; L[2] = ph[2];
                L[3] = dirs[3 * q]; L[4] = dirs[3 * q + 1]; L[5] = dirs[3 * q + 2];
            }
        }
        e = cudaMemcpy(dl.p, launch.data(), (size_t)m * nt * 6 * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(dstatus.p, 0, sizeof(unsigned));
        if (e != cudaSuccess) return cuda_fail(e, "mpf_rays_propagate");
        PropOut O{(long long*)dsteps.p, nullptr, nullptr, (unsigned*)dstatus.p, nullptr, (double*)dtraj.p, cap};
        e = (p->exact || hom) ? launch_propagate<true>(o->tree, C, P, (const double*)dl.p, m * nt, O, 0)
                     : launch_propagate<false>(o->tree, C, P, (const double*)dl.p, m * nt, O, 0);
        unsigned hs = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&hs, dstatus.p, sizeof(unsigned), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "mpf_rays_propagate: propagate");
        if (hs & 8u) return fail(MPF_BAD_INPUT, "mpf_rays_propagate: a trajectory is longer than capacity points");
        if (hs & 1u) rc = MPF_WARN_MAX_STEPS;
        rays::k_bundle<<<(unsigned)m, 128>>>((const double*)dtraj.p, (const long long*)dsteps.p, m, bp->count, cap,
                                             bp->interpolation, bp->amin, p->length, bp->angle, (double*)dout.p,
                                             (long long*)dsizes.p);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(sizes + b0, dsizes.p, (size_t)m * sizeof(long long), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(central + (size_t)b0 * cap * rays::kFileFields, dout.p, (size_t)m * cap * rays::kFileFields * sizeof(double),
                           cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "mpf_rays_propagate: bundles");
    }
    return rc;
}
