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
// The sources are sorted by the direction of their first ray (a 2-D Morton
// key of phi, theta) and every compaction keeps that order, so each warp
// traces 32 neighbouring rays: their gathers share cells and cache lines
// (rays of unrelated directions in one warp run several times slower).
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
#include "mpf_cat_device.cuh"

namespace mpf {

__global__ void k_cat_init(long long n, const double* __restrict__ src, int stride, CatRotation rot, int has_rot,
                           CatState* __restrict__ state, double* __restrict__ rows, uint32_t* __restrict__ key,
                           int* __restrict__ val, unsigned* __restrict__ count)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cat_init_one(i, src, stride, rot, has_rot, state, rows, key, val, count);
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
// bookkeeping of iterateNewtonMethod (catalogues.h:769-780): the listed
// source's outcome sets its continue, pending-bundle and re-trace flags.
__global__ void k_cat_update(long long m, int iteration, int traced_jacobian, CatConst K,
                             const int* __restrict__ list, CatState* __restrict__ state, double* __restrict__ rows,
                             const long long* __restrict__ steps, const double* __restrict__ rec,
                             int* __restrict__ cont, int* __restrict__ retrace_flag, int* __restrict__ pend,
                             unsigned long long* __restrict__ photon_steps)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > m) return;
    cont[j] = 0;   // continue flag, scanned into the next round's list (entry m closes the scan)
    pend[j] = 0;   // waiting for a bundle Jacobian before its Newton step
    if (j == m) return;
    const int s = list[j];
    const int r = cat_update(s, iteration, traced_jacobian, K, state, rows, steps[j], rec + (long long)kSourceFields * j,
                             photon_steps);
    if (r == kCatContinue) cont[j] = 1;
    else if (r == kCatPendBundle) pend[j] = 1;
    else if (r == kCatRetrace) retrace_flag[s] = 1;
}

// Jacobian of a converged source whose last ray was traced without it, or
// (jacobiantype = infinitesimal_born) the one of its Born ray.
__global__ void k_cat_jacobian(long long m, const int* __restrict__ list, const double* __restrict__ rec,
                               const long long* __restrict__ steps, double* __restrict__ rows,
                               unsigned long long* __restrict__ photon_steps, int born)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    cat_final_jacobian(rows + (long long)kCatalogueFields * list[j], rec + (long long)kSourceFields * j, steps[j],
                       photon_steps, born);
}

// Four bundle rays per listed source (Lensing::dbetadtheta, lensing.h:160-196)
// around its current launch direction, each with the single surface iref.
__global__ void k_cat_bundle_rays(long long nb, const int* __restrict__ srcs, const CatState* __restrict__ state,
                                  CatConst K, double* __restrict__ blaunch, double* __restrict__ bplanes,
                                  double* __restrict__ bki)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const CatState& S = state[srcs[k]];
    const double cp = cos(S.phi), sp = sin(S.phi), ct = cos(S.theta), st = sin(S.theta);
    const double tx = cp * st, ty = sp * st, tz = ct;
    const double e1x = -sp, e1y = cp;
    const double e2x = -cp * ct, e2y = -sp * ct, e2z = st;
    const double to = tan(K.openingmin);
    double* B = blaunch + 24 * k;
    for (int r = 0; r < 4; ++r) {
        B[6 * r] = 0.0; B[6 * r + 1] = 0.0; B[6 * r + 2] = 0.0;
        bplanes[4 * k + r] = S.iref;
        if (bki) {   // stop_bundle = "plane": the screen normal is the stop plane's normal
            bki[12 * k + 3 * r] = S.kx; bki[12 * k + 3 * r + 1] = S.ky; bki[12 * k + 3 * r + 2] = S.kz;
        }
    }
    B[3] = tx + to * e1x; B[4] = ty + to * e1y; B[5] = tz;
    B[9] = tx - to * e1x; B[10] = ty - to * e1y; B[11] = tz;
    B[15] = tx - to * e2x; B[16] = ty - to * e2y; B[17] = tz - to * e2z;
    B[21] = tx + to * e2x; B[22] = ty + to * e2y; B[23] = tz + to * e2z;
}

// The four-ray Jacobian at the source distance (lensing.h:198-334, one
// surface); false when a bundle ray ended before the surface (J = 42 42 1 0,
// or 42 42 1 3 for stop_bundle = "a").
__device__ bool cat_bundle_jacobian(const double* r4, const CatState& S, const CatConst& K, double* J)
{
    for (int r = 0; r < 4; ++r) {
        if (r4[r * kWideFields + 24] == 0.0) {
            J[0] = 42; J[1] = 42; J[2] = 1; J[3] = (K.stop_bundle == STOP_A) ? 3 : 0;
            return false;
        }
    }
    const double* r0 = r4;
    const double* r1 = r4 + kWideFields;
    const double* r2 = r4 + 2 * kWideFields;
    const double* r3 = r4 + 3 * kWideFields;
    double rh[3], rv[3];
    for (int d = 0; d < 3; ++d) {
        rh[d] = r0[2 + d] - r1[2 + d];
        rv[d] = r2[2 + d] - r3[2 + d];
    }
    const double phik = atan2(S.ky, S.kx);
    const double thetak = acos(S.kz / sqrt(S.kx * S.kx + S.ky * S.ky + S.kz * S.kz));
    const double cpk = cos(phik), spk = sin(phik), ctk = cos(thetak), stk = sin(thetak);
    const double to = tan(K.openingmin);
    const double d2 = 2 * S.dist * to;
    J[0] = (rh[0] * -spk + rh[1] * cpk) / d2;
    J[1] = (rv[0] * -spk + rv[1] * cpk) / d2;
    J[2] = (rh[0] * (-cpk * ctk) + rh[1] * (-spk * ctk) + rh[2] * stk) / (-d2);
    J[3] = (rv[0] * (-cpk * ctk) + rv[1] * (-spk * ctk) + rv[2] * stk) / (-d2);
    return true;
}

// Newton step of the sources that waited for their bundle Jacobian (round >= 5).
__global__ void k_cat_bundle_newton(long long nb, int iteration, CatConst K, const int* __restrict__ srcs,
                                    CatState* __restrict__ state, double* __restrict__ rows,
                                    const double* __restrict__ brec, int* __restrict__ cont_src)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const int s = srcs[k];
    CatState S = state[s];
    double* row = rows + (long long)kCatalogueFields * s;
    double J[4];
    const bool ok = cat_bundle_jacobian(brec + 4 * k * kWideFields, S, K, J);
    row[12] = J[0]; row[13] = J[1]; row[14] = J[2]; row[15] = J[3];
    if (!ok) {
        // catalogues.h:521-528 (the reference leaves column 5 unset there)
        row[2] = 42.0; row[3] = 42.0; row[4] = 22.0; row[5] = 0.0;
        return;
    }
    const double invdet = 1. / (J[0] * J[3] - J[1] * J[2]);
    double nphi, ntheta;
    newton_step(S, S.fx, S.fy, S.fz, J[3] * invdet, -J[1] * invdet, -J[2] * invdet, J[0] * invdet, nphi, ntheta);
    row[2] = nphi; row[3] = ntheta; row[4] = S.miss;
    if ((unsigned)iteration + 1u > (unsigned)K.max_iterations) {
        row[5] = 42.0;   // rejected
        return;
    }
    S.phi = nphi;
    S.theta = ntheta;
    state[s] = S;
    cont_src[s] = 1;
}

// Bundle Jacobian of the converged sources (catalogues.h:661-676); a failed
// bundle turns the source into a failure row as the reference does.
__global__ void k_cat_bundle_final(long long nb, CatConst K, const int* __restrict__ srcs,
                                   const CatState* __restrict__ state, double* __restrict__ rows,
                                   const double* __restrict__ brec)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const int s = srcs[k];
    double* row = rows + (long long)kCatalogueFields * s;
    double J[4];
    const bool ok = cat_bundle_jacobian(brec + 4 * k * kWideFields, state[s], K, J);
    row[12] = J[0]; row[13] = J[1]; row[14] = J[2]; row[15] = J[3];
    if (!ok) {
        row[2] = 42.0; row[3] = 42.0; row[4] = 22.0; row[5] = 0.0;
        row[6] = 0.0; row[8] = 0.0; row[9] = 0.0; row[10] = 0.0; row[11] = 0.0;
    }
}

// Next round's flags: the in-round continuations and the bundle Newton ones.
__global__ void k_merge_cont(long long m, const int* __restrict__ list, const int* __restrict__ cont_src,
                             int* __restrict__ cont)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    if (cont_src[list[j]]) cont[j] = 1;
}

// Stable LSD radix sort of (key, value) pairs: 4-bit digits, each thread
// walks one tile of kSortTile consecutive entries in order.
constexpr int kSortTile = 256;

__global__ void k_sort_hist(const uint32_t* __restrict__ key, long long n, int shift, int* __restrict__ hist,
                            long long ntiles)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    int h[16];
    for (int d = 0; d < 16; ++d) h[d] = 0;
    const long long e = min(n, (t + 1) * kSortTile);
    for (long long i = t * kSortTile; i < e; ++i) ++h[(key[i] >> shift) & 15u];
    for (int d = 0; d < 16; ++d) hist[d * ntiles + t] = h[d];
}

__global__ void k_sort_scatter(const uint32_t* __restrict__ key, const int* __restrict__ val, long long n, int shift,
                               const int* __restrict__ off, long long ntiles, uint32_t* __restrict__ key2,
                               int* __restrict__ val2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    int o[16];
    for (int d = 0; d < 16; ++d) o[d] = off[d * ntiles + t];
    const long long e = min(n, (t + 1) * kSortTile);
    for (long long i = t * kSortTile; i < e; ++i) {
        const uint32_t k = key[i];
        const int j = o[(k >> shift) & 15u]++;
        key2[j] = k;
        val2[j] = val[i];
    }
}

// Order-keeping compaction: scan holds the exclusive prefix sum of the flags
// over m + 1 entries.
__global__ void k_compact(long long m, const int* __restrict__ from, const int* __restrict__ scan, int* __restrict__ to)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    if (scan[j + 1] > scan[j]) to[scan[j]] = from[j];
}

// Flags of a list's entries from a per-source flag array (entry m = 0).
__global__ void k_list_flags(long long m, const int* __restrict__ list, const int* __restrict__ per_source,
                             int* __restrict__ flags)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > m) return;
    flags[j] = (j < m) ? per_source[list[j]] : 0;
}

namespace {
unsigned blocks(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// Scratch of one call, stream-ordered (cudaMallocAsync / cudaFreeAsync), so
// that calls on different streams neither wait for one another nor for the
// whole device when they free.
struct CatBuffers {
    void* p[21] = {};
    cudaStream_t stream = nullptr;
    ~CatBuffers()
    {
        for (void* q : p)
            if (q) cudaFreeAsync(q, stream);
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
    // work items carry the source index times two: up to 2^30 sources per call
    if (catalogue_persistent_applies(K, exact, order) && n < (1ll << 30)) {
        bool queue_error = false;
        const cudaError_t pe = catalogue_newton_persistent(T, Cs, K, rot, order, nsteps, n, d_src, stride, d_rows, stats,
                                                           h_status, &queue_error, stream);
        if (pe == cudaSuccess && queue_error) *h_status |= kCatQueueError;
        return pe;
    }
    const int tpb = 128;
    const long long ntiles = (n + kSortTile - 1) / kSortTile;
    CatBuffers B;
    B.stream = stream;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](int k, size_t bytes) -> void* {
        if (e != cudaSuccess) return nullptr;
        e = cudaMallocAsync(&B.p[k], bytes, stream);
        return (e == cudaSuccess) ? B.p[k] : nullptr;
    };
    CatState* state = (CatState*)alloc(0, (size_t)n * sizeof(CatState));
    int* act0 = (int*)alloc(1, (size_t)n * sizeof(int));
    int* act1 = (int*)alloc(2, (size_t)n * sizeof(int));
    int* rflag = (int*)alloc(3, (size_t)n * sizeof(int));
    unsigned* counters = (unsigned*)alloc(4, 8 * sizeof(unsigned));   // [0] valid sources, [3] status
    unsigned long long* psteps = (unsigned long long*)alloc(5, 2 * sizeof(unsigned long long));
    double* launch = (double*)alloc(6, (size_t)n * 6 * sizeof(double));
    double* radius = (double*)alloc(7, (size_t)n * sizeof(double));
    double* rec = (double*)alloc(8, (size_t)n * kSourceFields * sizeof(double));
    long long* steps = (long long*)alloc(9, (size_t)n * sizeof(long long));
    uint32_t* key0 = (uint32_t*)alloc(10, (size_t)n * sizeof(uint32_t));
    uint32_t* key1 = (uint32_t*)alloc(11, (size_t)n * sizeof(uint32_t));
    int* scan = (int*)alloc(12, (size_t)(std::max<long long>(n, 16 * ntiles) + 1) * sizeof(int));
    int* pend = (int*)alloc(13, (size_t)(n + 1) * sizeof(int));
    // bundle Jacobian (jacobiantype = bundle): four rays per source in a pass
    int *plist = nullptr, *cont_src = nullptr;
    double *blaunch = nullptr, *bplanes = nullptr, *brec = nullptr, *bki = nullptr;
    long long* bsteps = nullptr;
    if (K.bundle) {
        plist = (int*)alloc(14, (size_t)n * sizeof(int));
        cont_src = (int*)alloc(15, (size_t)n * sizeof(int));
        blaunch = (double*)alloc(16, (size_t)n * 24 * sizeof(double));
        bplanes = (double*)alloc(17, (size_t)n * 4 * sizeof(double));
        brec = (double*)alloc(18, (size_t)n * 4 * kWideFields * sizeof(double));
        bsteps = (long long*)alloc(19, (size_t)n * 4 * sizeof(long long));
        if (K.stop_bundle == STOP_PLANE) bki = (double*)alloc(20, (size_t)n * 12 * sizeof(double));
    }
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(psteps, 0, 2 * sizeof(unsigned long long), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(rflag, 0, (size_t)n * sizeof(int), stream);
    if (e != cudaSuccess) return e;
    CatRotation R{};
    if (rot) R = *rot;
    k_cat_init<<<blocks(n, tpb), tpb, 0, stream>>>(n, d_src, stride, R, rot ? 1 : 0, state, d_rows, key0, act0, counters);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    stats->launches = 1;
    // sources in radius-bin and direction order; the unreachable ones (key 0xffffffff) sort last
    {
        uint32_t *ka = key0, *kb = key1;
        int *va = act0, *vb = act1;
        for (int shift = 0; shift < 32; shift += 4) {
            k_sort_hist<<<blocks(ntiles, tpb), tpb, 0, stream>>>(ka, n, shift, scan, ntiles);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            exclusive_scan(scan, 16 * ntiles, stream);
            k_sort_scatter<<<blocks(ntiles, tpb), tpb, 0, stream>>>(ka, va, n, shift, scan, ntiles, kb, vb);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            std::swap(ka, kb);
            std::swap(va, vb);
            stats->launches += 2;
        }
        // eight passes: the sorted values are back in act0
    }
    unsigned m = 0;
    if ((e = cudaMemcpyAsync(&m, counters, sizeof(unsigned), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    const unsigned m_valid = m;
    // act0 keeps the valid sources in that order (for the re-trace); the
    // rounds compact between act1 and the key buffer, free after the sort
    int* sorted = act0;
    int* cur = act1;
    int* nxt = reinterpret_cast<int*>(key0);
    if ((e = cudaMemcpyAsync(cur, sorted, (size_t)m * sizeof(int), cudaMemcpyDeviceToDevice, stream)) != cudaSuccess) return e;

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
    // the bundle rays: their own stop criterion and one surface each
    PropParams Pb = P;
    Pb.ray_stop = nullptr;
    Pb.stop_kind = K.stop_bundle;
    Pb.ray_planes = bplanes;
    Pb.ray_ki = bki;
    Pb.wide = 1;
    Pb.jacobian = 0;
    const PropOut Ob{bsteps, nullptr, brec, counters + 3, nullptr};
    auto bundle_pass = [&](long long nb, const int* srcs) -> cudaError_t {
        k_cat_bundle_rays<<<blocks(nb, tpb), tpb, 0, stream>>>(nb, srcs, state, K, blaunch, bplanes, bki);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        stats->rays += 4 * nb;
        stats->launches += 2;
        return exact ? launch_propagate<true>(T, Cs, Pb, blaunch, 4 * nb, Ob, stream)
                     : launch_propagate<false>(T, Cs, Pb, blaunch, 4 * nb, Ob, stream);
    };
    for (int it = 0; it <= K.max_iterations && m > 0; ++it) {
        // the infinitesimal Jacobian serves the Newton steps of rounds 3 and up
        // (3 and 4 before the bundle rounds); round 2 traces it too, so that
        // the sources converging there (most of them) need no re-trace for
        // their final Jacobian
        const int jac = K.bundle ? ((it >= 3 && it < 5) ? 1 : 0) : K.born ? ((it >= 3) ? 1 : 0) : ((it >= 2) ? 1 : 0);
        P.jacobian = jac;
        // round 2 also re-traces, with the Jacobian, the sources that converged
        // in rounds 0 and 1 (appended after the active ones): their final
        // Jacobian then costs no launch of its own at the end
        long long nre = 0;
        if (it == 2 && !K.bundle && !K.born) {
            k_list_flags<<<blocks((long long)m_valid + 1, tpb), tpb, 0, stream>>>(m_valid, sorted, rflag, scan);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            nre = exclusive_scan(scan, (int64_t)m_valid + 1, stream);
            if (nre > 0) {
                k_compact<<<blocks(m_valid, tpb), tpb, 0, stream>>>(m_valid, sorted, scan, cur + m);
                if ((e = cudaMemsetAsync(rflag, 0, (size_t)n * sizeof(int), stream)) != cudaSuccess) return e;
            }
            stats->launches += 2;
        }
        const long long mt = (long long)m + nre;
        k_cat_rays<<<blocks(mt, tpb), tpb, 0, stream>>>(mt, cur, state, launch, radius);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = exact ? launch_propagate<true>(T, Cs, P, launch, mt, O, stream) : launch_propagate<false>(T, Cs, P, launch, mt, O, stream);
        if (e != cudaSuccess) return e;
        if (nre > 0) {
            k_cat_jacobian<<<blocks(nre, tpb), tpb, 0, stream>>>(nre, cur + m, rec + (long long)kSourceFields * m, steps + m,
                                                                  d_rows, psteps, 0);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            stats->rays += nre;
            stats->launches += 1;
        }
        k_cat_update<<<blocks(m + 1, tpb), tpb, 0, stream>>>(m, it, jac, K, cur, state, d_rows, steps, rec, scan, rflag,
                                                              pend, psteps);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (K.bundle && it >= 5) {
            const int64_t npend = exclusive_scan(pend, (int64_t)m + 1, stream);
            if (npend > 0) {
                k_compact<<<blocks(m, tpb), tpb, 0, stream>>>(m, cur, pend, plist);
                if ((e = cudaMemsetAsync(cont_src, 0, (size_t)n * sizeof(int), stream)) != cudaSuccess) return e;
                if ((e = bundle_pass(npend, plist)) != cudaSuccess) return e;
                k_cat_bundle_newton<<<blocks(npend, tpb), tpb, 0, stream>>>(npend, it, K, plist, state, d_rows, brec,
                                                                            cont_src);
                k_merge_cont<<<blocks(m, tpb), tpb, 0, stream>>>(m, cur, cont_src, scan);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                stats->launches += 3;
            }
        }
        const int64_t next_m = exclusive_scan(scan, (int64_t)m + 1, stream);
        k_compact<<<blocks(m, tpb), tpb, 0, stream>>>(m, cur, scan, nxt);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        stats->rays += m;
        stats->iterations = it + 1;
        stats->launches += 4;
        m = (unsigned)next_m;
        std::swap(cur, nxt);
    }
    // Jacobian of the sources that converged in rounds traced without it,
    // re-traced in radius-bin and direction order
    k_list_flags<<<blocks((long long)m_valid + 1, tpb), tpb, 0, stream>>>(m_valid, sorted, rflag, scan);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int64_t r = exclusive_scan(scan, (int64_t)m_valid + 1, stream);
    stats->launches += 1;
    if (r > 0 && K.bundle) {
        // converged sources: the four-ray Jacobian
        k_compact<<<blocks(m_valid, tpb), tpb, 0, stream>>>(m_valid, sorted, scan, cur);
        if ((e = bundle_pass(r, cur)) != cudaSuccess) return e;
        k_cat_bundle_final<<<blocks(r, tpb), tpb, 0, stream>>>(r, K, cur, state, d_rows, brec);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        stats->launches += 2;
    } else if (r > 0) {
        k_compact<<<blocks(m_valid, tpb), tpb, 0, stream>>>(m_valid, sorted, scan, cur);
        P.jacobian = 1;
        k_cat_rays<<<blocks(r, tpb), tpb, 0, stream>>>(r, cur, state, launch, radius);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (K.born) {
            // the Born ray of the converged direction to the source radius
            // (catalogues.h:670-673)
            PropParams Pn = P;
            Pn.homogeneous = 2;
            e = exact ? launch_propagate<true>(T, Cs, Pn, launch, r, O, stream) : launch_propagate<false>(T, Cs, Pn, launch, r, O, stream);
        } else {
            e = exact ? launch_propagate<true>(T, Cs, P, launch, r, O, stream) : launch_propagate<false>(T, Cs, P, launch, r, O, stream);
        }
        if (e != cudaSuccess) return e;
        k_cat_jacobian<<<blocks(r, tpb), tpb, 0, stream>>>(r, cur, rec, steps, d_rows, psteps, K.born);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        stats->rays += r;
        stats->launches += 4;
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
