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
__global__ void k_fill_maps(long long n, int nz, MapSpec M, const double* __restrict__ launch,
                            const double* __restrict__ rec, float* __restrict__ maps, long long row_stride,
                            long long col0)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * nz) return;
    const long long j = t % n;
    const int iz = (int)(t / n);
    const double* o = rec + ((long long)j * nz + iz) * kPlaneFields;
    float* out = maps + (long long)M.nmaps * iz * row_stride + col0 + j;
    if (o[19] == 0.0) {
        for (int r = 0; r < M.nmaps; ++r) out[(long long)r * row_stride] = 0.0f;
        return;
    }
    const double* H = M.homogeneous[iz];   // t chi lambda a z of the FLRW ray at the surface
    int row = 0;
    for (int q = 0; q < M.ncomp; ++q) {
        switch (M.comp[q]) {
        case 0: {
            const double a11 = o[6], a12 = o[7], a22 = o[8];
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
    for (long long c0 = 0; e == cudaSuccess && c0 < npix; c0 += cap) {
        const long long m = (npix - c0 < cap) ? npix - c0 : cap;
        k_pix_launch<<<blocks(m, 128), 128, 0, stream>>>(m, nside, d_pixels + c0, launch);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        e = exact ? launch_propagate<true>(T, C, P, launch, m, O, stream) : launch_propagate<false>(T, C, P, launch, m, O, stream);
        if (e != cudaSuccess) break;
        k_fill_maps<<<blocks(m * nz, 128), 128, 0, stream>>>(m, nz, M, launch, rec, d_maps, npix, c0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_status, status, sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (launch) cudaFree(launch);
    if (rec) cudaFree(rec);
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
