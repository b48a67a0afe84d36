// HEALPix map filling on the device: the per-pixel body of Hmaps::FillMap
// (src/hmaps.h:583-832, jacobiantype = "infinitesimal") for a whole set of
// pixels: RING pixel -> direction, one batched ray launch through the
// propagate kernel (surface records with the fused Jacobian), and the map
// rows written as float, one row of npix values per (surface, component row)
// in the reference's map vector order map[nmaps * iz + row][pixel].
#include <cmath>
#include <cstring>

#include "mpf_internal.h"
#include "mpf_maps.h"

namespace mpf {

// RING-scheme pixel centre (Gorski et al. 2005, ApJ 622, 759, eqs. 4-10),
// the reference's pix2vec_ring call (hmaps.h:599).
__device__ void pix2vec_ring(long long nside, long long ipix, double* v)
{
    const double ns = (double)nside;
    const long long ncap = 2 * nside * (nside - 1);
    const long long npix = 12 * nside * nside;
    const double pi = 3.14159265358979323846;
    double z, phi;
    if (ipix < ncap) {                       // north polar cap
        long long ir = (1 + (long long)sqrt((double)(1 + 2 * ipix))) / 2;
        while (ir > 1 && 2 * ir * (ir - 1) > ipix) --ir;
        while (2 * (ir + 1) * ir <= ipix) ++ir;
        const long long iphi = ipix - 2 * ir * (ir - 1) + 1;
        z = 1.0 - (double)(ir * ir) / (3.0 * ns * ns);
        phi = ((double)iphi - 0.5) * (pi / (2.0 * (double)ir));
    } else if (ipix < npix - ncap) {         // equatorial belt
        const long long ip = ipix - ncap;
        const long long iring = ip / (4 * nside) + nside;
        const long long iphi = ip % (4 * nside) + 1;
        const double fodd = ((iring + nside) & 1) ? 1.0 : 0.5;
        z = (2.0 * ns - (double)iring) * 2.0 / (3.0 * ns);
        phi = ((double)iphi - fodd) * (pi / (2.0 * ns));
    } else {                                 // south polar cap
        const long long ip = npix - ipix;
        long long ir = (1 + (long long)sqrt((double)(2 * ip - 1))) / 2;
        while (ir > 1 && 2 * ir * (ir - 1) >= ip) --ir;
        while (2 * (ir + 1) * ir < ip) ++ir;
        const long long iphi = 4 * ir + 1 - (ip - 2 * ir * (ir - 1));
        z = -1.0 + (double)(ir * ir) / (3.0 * ns * ns);
        phi = ((double)iphi - 0.5) * (pi / (2.0 * (double)ir));
    }
    const double st = sqrt((1.0 - z) * (1.0 + z));
    v[0] = st * cos(phi);
    v[1] = st * sin(phi);
    v[2] = z;
}

__global__ void k_pix_launch(long long n, long long nside, const long long* __restrict__ pixels,
                             double* __restrict__ launch)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[3];
    pix2vec_ring(nside, pixels[i], v);
    double* L = launch + 6 * i;
    L[0] = 0.0; L[1] = 0.0; L[2] = 0.0;    // the observer (hmaps.cpp: origin of the cone octree)
    L[3] = v[0]; L[4] = v[1]; L[5] = v[2];
}

// One thread per (pixel, surface): the map rows of hmaps.h:716-829.
// rec_fields: stride of the surface records (unused with only_born); jac: the
// bundle Jacobians (n x nz x 4: a11 a12 a21 a22) or null for the
// infinitesimal one; born: the Born rays' wide surface records (n x nz x 32)
// or null.
__global__ void k_fill_maps(long long n, int nz, MapSpec M, const double* __restrict__ launch,
                            const double* __restrict__ rec, int rec_fields, const double* __restrict__ jac,
                            const double* __restrict__ born, float* __restrict__ maps, long long row_stride,
                            long long col0)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * nz) return;
    const long long j = t % n;
    const int iz = (int)(t / n);
    const double* o = M.only_born ? nullptr : rec + ((long long)j * nz + iz) * rec_fields;
    const double* bj = jac ? jac + ((long long)j * nz + iz) * 4 : nullptr;
    const double* ob = born ? born + ((long long)j * nz + iz) * kWideFields : nullptr;
    float* out = maps + (long long)M.nmaps * iz * row_stride + col0 + j;
    // a Born ray that took no step, an unusable crossing of the traced ray, or
    // a bundle Jacobian flagged 42, zeroes the surface (hmaps.h:719-738)
    if ((ob && ob[19] == 0.0) || (o && o[19] == 0.0) || (bj && bj[0] == 42.0)) {
        for (int r = 0; r < M.nmaps; ++r) out[(long long)r * row_stride] = 0.0f;
        return;
    }
    const double* H = M.homogeneous[iz];   // t chi lambda a z of the FLRW ray at the surface
    int row = 0;
    for (int q = 0; q < M.ncomp; ++q) {
        switch (M.comp[q]) {
        case 0: {
            if (bj) {
                // bundle: image rotation w first (hmaps.h:725-733), five rows
                const double a11 = bj[0], a12 = bj[1], a21 = bj[2], a22 = bj[3];
                const double w = -atan2(a12 - a21, a11 + a22);
                out[(long long)(row + 0) * row_stride] = (float)(1 - (a11 + a22) * 0.5 / cos(w));
                out[(long long)(row + 1) * row_stride] = (float)(-0.5 * (cos(w) * (a11 - a22) + sin(w) * (a12 + a21)));
                out[(long long)(row + 2) * row_stride] = (float)(-0.5 * (cos(w) * (a12 + a21) + sin(w) * (a22 - a11)));
                out[(long long)(row + 3) * row_stride] = (float)w;
                out[(long long)(row + 4) * row_stride] = (float)(a11 * a22 - a12 * a21);
                row += 5;
                break;
            }
            const double a11 = o[6], a12 = o[7], a22 = o[8];
            out[(long long)(row + 0) * row_stride] = (float)(1 - (a11 + a22) * 0.5);
            out[(long long)(row + 1) * row_stride] = (float)(-0.5 * (a11 - a22));
            out[(long long)(row + 2) * row_stride] = (float)(-a12);
            out[(long long)(row + 3) * row_stride] = (float)(a11 * a22 - a12 * a12);
            row += 4;
            break;
        }
        case 1: {
            // lensing_born (hmaps.h:771-785)
            const double a11 = ob[6], a12 = ob[7], a22 = ob[8];
            out[(long long)(row + 0) * row_stride] = (float)(1 - (a11 + a22) * 0.5);
            out[(long long)(row + 1) * row_stride] = (float)(-0.5 * (a11 - a22));
            out[(long long)(row + 2) * row_stride] = (float)(-a12);
            out[(long long)(row + 3) * row_stride] = (float)(a11 * a22 - a12 * a12);
            row += 4;
            break;
        }
        case 2: out[(long long)row++ * row_stride] = (float)(o[12] / H[1] - 1); break;
        case 3: out[(long long)row++ * row_stride] = (float)(o[13] / H[2] - 1); break;
        case 4: out[(long long)row++ * row_stride] = (float)(o[9] / H[0] - 1); break;
        case 5: out[(long long)row++ * row_stride] = (float)(o[10] / H[3] - 1); break;
        case 6: out[(long long)row++ * row_stride] = (float)(o[11] / H[4] - 1); break;
        case 7: out[(long long)row++ * row_stride] = (float)(o[14] / H[1] - 1); break;
        case 8: out[(long long)row++ * row_stride] = (float)o[15]; break;
        case 9: out[(long long)row++ * row_stride] = (float)o[16]; break;
        case 10: out[(long long)row++ * row_stride] = (float)o[18]; break;
        case 11: out[(long long)row++ * row_stride] = (float)o[0]; break;
        case 12: out[(long long)row++ * row_stride] = (float)o[17]; break;
        case 13: {
            const double* L = launch + 6 * j;
            const double phi = atan2(L[4], L[3]);
            const double theta = acos(L[5]);
            const double beta1 = atan2(o[3], o[2]);
            const double beta2 = acos(o[4] / o[5]);
            out[(long long)(row + 0) * row_stride] = (float)(phi - beta1);
            out[(long long)(row + 1) * row_stride] = (float)(theta - beta2);
            row += 2;
            break;
        }
        default: break;
        }
    }
}

// Bundle rays of each pixel (Lensing::dbetadtheta, lensing.h:160-196) and
// their surfaces from the central ray's crossings (hmaps.h:653-693):
// kiTargets (the interpolated direction, or position), the stop_bundle value
// at each surface and the surface distance.
__global__ void k_bundle_prepare(long long n, int nz, MapSpec M, const double* __restrict__ planes,
                                 const double* __restrict__ launch, const double* __restrict__ rec,
                                 double* __restrict__ blaunch, double* __restrict__ bplanes, double* __restrict__ ki,
                                 double* __restrict__ dist, double* __restrict__ bki)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int iz = 0; iz < nz; ++iz) {
        const double* o = rec + ((long long)j * nz + iz) * kWideFields;
        double* k = ki + ((long long)j * nz + iz) * 3;
        const bool found = o[24] != 0.0;
        if (M.plane_sachs && found) {
            k[0] = o[21]; k[1] = o[22]; k[2] = o[23];
        } else {
            k[0] = o[2]; k[1] = o[3]; k[2] = o[4];
        }
        dist[(long long)j * nz + iz] = o[5];
        double v;
        switch (M.stop_bundle) {
        case STOP_LAMBDA: v = o[13]; break;
        case STOP_R: v = o[12]; break;
        case STOP_REDSHIFT: v = o[11]; break;
        case STOP_A: v = o[10]; break;
        case STOP_T: v = o[9]; break;
        case STOP_PLANE: v = k[0] * o[2] + k[1] * o[3] + k[2] * o[4]; break;   // kiTarget . posTarget
        default: v = o[11];
        }
        // a surface the central ray never reached has no interpolated value
        // (the reference reads past the trajectory there); its own value stands in
        if (!found) v = planes[iz];
        for (int r = 0; r < 4; ++r) {
            bplanes[(4 * j + r) * nz + iz] = v;
            if (bki)
                for (int d = 0; d < 3; ++d) bki[((4 * j + r) * nz + iz) * 3 + d] = k[d];
        }
    }
    // the screen around the pixel direction
    const double* L = launch + 6 * j;
    const double phi = atan2(L[4], L[3]), theta = acos(L[5]);
    const double cp = cos(phi), sp = sin(phi), ct = cos(theta), st = sin(theta);
    const double tx = cp * st, ty = sp * st, tz = ct;
    const double e1x = -sp, e1y = cp;
    const double e2x = -cp * ct, e2y = -sp * ct, e2z = st;
    const double to = tan(M.openingmin);
    double* B = blaunch + 24 * j;
    for (int r = 0; r < 4; ++r) { B[6 * r] = 0.0; B[6 * r + 1] = 0.0; B[6 * r + 2] = 0.0; }
    B[3] = tx + to * e1x; B[4] = ty + to * e1y; B[5] = tz;
    B[9] = tx - to * e1x; B[10] = ty - to * e1y; B[11] = tz;
    B[15] = tx - to * e2x; B[16] = ty - to * e2y; B[17] = tz - to * e2z;
    B[21] = tx + to * e2x; B[22] = ty + to * e2y; B[23] = tz + to * e2z;
}

// Finite-difference Jacobian of the four bundle rays at each surface
// (lensing.h:198-334).  A ray that ended before a surface flags the
// Jacobians with 42 as the reference does (all surfaces; for stop_bundle =
// "a" only that surface).
__global__ void k_bundle_jacobian(long long n, int nz, MapSpec M, const double* __restrict__ brec,
                                  const double* __restrict__ ki, const double* __restrict__ dist,
                                  double* __restrict__ jac)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double* J = jac + (long long)j * nz * 4;
    for (int q = 0; q < 4 * nz; ++q) J[q] = 0.0;
    for (int r = 0; r < 4; ++r) {
        for (int iz = 0; iz < nz; ++iz) {
            if (brec[((4 * j + r) * nz + iz) * kWideFields + 24] != 0.0) continue;
            if (M.stop_bundle == STOP_A) {
                J[4 * iz] = 42; J[4 * iz + 1] = 42; J[4 * iz + 2] = 1; J[4 * iz + 3] = 3;
            } else {
                for (int q = 0; q < nz; ++q) { J[4 * q] = 42; J[4 * q + 1] = 42; J[4 * q + 2] = 1; J[4 * q + 3] = 0; }
            }
            return;
        }
    }
    const double to = tan(M.openingmin);
    for (int iz = 0; iz < nz; ++iz) {
        const double* r0 = brec + ((4 * j + 0) * nz + iz) * kWideFields;
        const double* r1 = brec + ((4 * j + 1) * nz + iz) * kWideFields;
        const double* r2 = brec + ((4 * j + 2) * nz + iz) * kWideFields;
        const double* r3 = brec + ((4 * j + 3) * nz + iz) * kWideFields;
        double rh[3], rv[3];
        for (int d = 0; d < 3; ++d) {
            rh[d] = r0[2 + d] - r1[2 + d];
            rv[d] = r2[2 + d] - r3[2 + d];
        }
        const double* k = ki + ((long long)j * nz + iz) * 3;
        const double phik = atan2(k[1], k[0]);
        const double thetak = acos(k[2] / sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]));
        const double cpk = cos(phik), spk = sin(phik), ctk = cos(thetak), stk = sin(thetak);
        const double d2 = 2 * dist[(long long)j * nz + iz] * to;
        J[4 * iz + 0] = (rh[0] * -spk + rh[1] * cpk) / d2;
        J[4 * iz + 1] = (rv[0] * -spk + rv[1] * cpk) / d2;
        J[4 * iz + 2] = (rh[0] * (-cpk * ctk) + rh[1] * (-spk * ctk) + rh[2] * stk) / (-d2);
        J[4 * iz + 3] = (rv[0] * (-cpk * ctk) + rv[1] * (-spk * ctk) + rv[2] * stk) / (-d2);
    }
}

namespace {
unsigned blocks(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }
}  // namespace

cudaError_t hmaps_fill(const DevTree& T, const DevCosmo& C, const PropParams& P, bool exact, long long nside,
                       long long npix, const long long* d_pixels, const MapSpec& M, float* d_maps, long long chunk,
                       unsigned* h_status, cudaStream_t stream)
{
    *h_status = 0;
    if (npix <= 0) return cudaSuccess;
    const int nz = P.nplanes;
    const long long cap = (chunk > 0 && chunk < npix) ? chunk : npix;
    double *launch = nullptr, *rec = nullptr;
    long long* steps = nullptr;
    unsigned* status = nullptr;
    cudaError_t e = cudaMalloc(&launch, (size_t)cap * 6 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&rec, (size_t)cap * nz * kPlaneFields * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&steps, (size_t)cap * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(unsigned), stream);
    PropOut O{steps, nullptr, rec, status, nullptr};
    // lensing_born: one Born ray per pixel (hmaps.h:706-712) with radius
    // surfaces at the FLRW distances of the map surfaces (wide records)
    double* brn = nullptr;
    long long* brn_steps = nullptr;
    PropParams Pn = P;
    if (M.born) {
        if (e == cudaSuccess) e = cudaMalloc(&brn, (size_t)cap * nz * kWideFields * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&brn_steps, (size_t)cap * sizeof(long long));
        Pn.homogeneous = 2;
        Pn.stop_kind = STOP_R;
        Pn.jacobian = 1;
        Pn.wide = 1;
        Pn.direct = 0;
        Pn.ray_planes = nullptr;
        Pn.ray_ki = nullptr;
        for (int iz = 0; iz < nz; ++iz) Pn.planes[iz] = M.homogeneous[iz][1];
        Pn.stop_ref = M.homogeneous[nz - 1][1];
    }
    const PropOut On{brn_steps, nullptr, brn, status, nullptr};
    auto born_pass = [&](long long m) -> cudaError_t {
        if (!M.born) return cudaSuccess;
        return exact ? launch_propagate<true>(T, C, Pn, launch, m, On, stream) : launch_propagate<false>(T, C, Pn, launch, m, On, stream);
    };
    // (lensing_born alone traces neither the central nor the bundle rays)
    for (long long c0 = 0; (!M.bundle || M.only_born) && e == cudaSuccess && c0 < npix; c0 += cap) {
        const long long m = (npix - c0 < cap) ? npix - c0 : cap;
        k_pix_launch<<<blocks(m, 128), 128, 0, stream>>>(m, nside, d_pixels + c0, launch);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if (!M.only_born) {
            e = exact ? launch_propagate<true>(T, C, P, launch, m, O, stream) : launch_propagate<false>(T, C, P, launch, m, O, stream);
            if (e != cudaSuccess) break;
        }
        if ((e = born_pass(m)) != cudaSuccess) break;
        k_fill_maps<<<blocks(m * nz, 128), 128, 0, stream>>>(m, nz, M, launch, rec, kPlaneFields, nullptr, brn, d_maps,
                                                               npix, c0);
        e = cudaGetLastError();
    }
    if (M.bundle && !M.only_born && e == cudaSuccess) {
        // central rays with wide records, then four bundle rays per pixel to
        // their own stop_bundle surfaces, then the Jacobians and the rows
        double *wrec = nullptr, *blaunch = nullptr, *bplanes = nullptr, *brec = nullptr, *ki = nullptr, *dist = nullptr,
               *jac = nullptr, *dplanes = nullptr, *bki = nullptr;
        long long* bsteps = nullptr;
        e = cudaMalloc(&wrec, (size_t)cap * nz * kWideFields * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&blaunch, (size_t)cap * 24 * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&bplanes, (size_t)cap * 4 * nz * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&brec, (size_t)cap * 4 * nz * kWideFields * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&ki, (size_t)cap * nz * 3 * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&dist, (size_t)cap * nz * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&jac, (size_t)cap * nz * 4 * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&bsteps, (size_t)cap * 4 * sizeof(long long));
        if (e == cudaSuccess) e = cudaMalloc(&dplanes, (size_t)nz * sizeof(double));
        // stop_bundle = plane: each bundle ray's surfaces are planes of normal kiTarget
        if (e == cudaSuccess && M.stop_bundle == STOP_PLANE) e = cudaMalloc(&bki, (size_t)cap * 4 * nz * 3 * sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpyAsync(dplanes, P.planes, (size_t)nz * sizeof(double), cudaMemcpyHostToDevice, stream);
        PropParams Pc = P;
        Pc.wide = 1;
        Pc.jacobian = 0;
        PropParams Pb = P;
        Pb.wide = 1;
        Pb.jacobian = 0;
        Pb.stop_kind = M.stop_bundle;
        Pb.ray_planes = bplanes;
        Pb.ray_ki = bki;
        const PropOut Oc{steps, nullptr, wrec, status, nullptr};
        const PropOut Ob{bsteps, nullptr, brec, status, nullptr};
        for (long long c0 = 0; e == cudaSuccess && c0 < npix; c0 += cap) {
            const long long m = (npix - c0 < cap) ? npix - c0 : cap;
            k_pix_launch<<<blocks(m, 128), 128, 0, stream>>>(m, nside, d_pixels + c0, launch);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            e = exact ? launch_propagate<true>(T, C, Pc, launch, m, Oc, stream) : launch_propagate<false>(T, C, Pc, launch, m, Oc, stream);
            if (e != cudaSuccess) break;
            k_bundle_prepare<<<blocks(m, 128), 128, 0, stream>>>(m, nz, M, dplanes, launch, wrec, blaunch, bplanes, ki, dist,
                                                                  bki);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            e = exact ? launch_propagate<true>(T, C, Pb, blaunch, 4 * m, Ob, stream)
                      : launch_propagate<false>(T, C, Pb, blaunch, 4 * m, Ob, stream);
            if (e != cudaSuccess) break;
            k_bundle_jacobian<<<blocks(m, 128), 128, 0, stream>>>(m, nz, M, brec, ki, dist, jac);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            if ((e = born_pass(m)) != cudaSuccess) break;
            k_fill_maps<<<blocks(m * nz, 128), 128, 0, stream>>>(m, nz, M, launch, wrec, kWideFields, jac, brn, d_maps, npix,
                                                                   c0);
            e = cudaGetLastError();
        }
        cudaStreamSynchronize(stream);
        for (void* q : {(void*)wrec, (void*)blaunch, (void*)bplanes, (void*)brec, (void*)ki, (void*)dist, (void*)jac,
                        (void*)bsteps, (void*)dplanes, (void*)bki})
            if (q) cudaFree(q);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_status, status, sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (launch) cudaFree(launch);
    if (rec) cudaFree(rec);
    if (brn) cudaFree(brn);
    if (brn_steps) cudaFree(brn_steps);
    if (steps) cudaFree(steps);
    if (status) cudaFree(status);
    return e;
}

// Device directions of RING pixels (tests and callers that launch their own rays).
cudaError_t pix2vec_device(long long nside, long long n, const long long* d_pixels, double* d_launch, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    k_pix_launch<<<blocks(n, 128), 128, 0, stream>>>(n, nside, d_pixels, d_launch);
    return cudaGetLastError();
}

}  // namespace mpf
