// Map filling driver (mpf_maps.cu), called by the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "mpf_device.cuh"
#include "mpf_propagate.cuh"

namespace mpf {

constexpr int kMaxMapComponents = 16;

struct MapSpec {
    int ncomp;
    int comp[kMaxMapComponents];      // index_components of hmaps.cpp (0 lensing, 1 lensing_born, 2-13 the others)
    int nmaps;                        // rows per surface
    double homogeneous[kMaxPlanes][5];   // per surface: t chi lambda a z of the FLRW ray
    // jacobiantype = "bundle" (Lensing::dbetadtheta): 4 rays per pixel
    int bundle;
    int plane_sachs;                  // screen normal: interpolated direction (1) or position (0)
    int stop_bundle;                  // StopKind of the bundle rays' surfaces
    double openingmin;                // bundle opening (radians)
    // lensing_born: a Born ray per pixel (homogeneous field on the octree's
    // levels, Jacobian at the FLRW surface radii); only_born: no traced ray
    int born;
    int only_born;
};

// d_pixels: npix RING pixel ids on the device; d_maps: nmaps * nplanes rows of
// npix floats on the device.  Rays are traced `chunk` pixels at a time
// (<= 0: all at once).  Synchronises `stream` at the end.
cudaError_t hmaps_fill(const DevTree& T, const DevCosmo& C, const PropParams& P, bool exact, long long nside,
                       long long npix, const long long* d_pixels, const MapSpec& M, float* d_maps, long long chunk,
                       unsigned* h_status, cudaStream_t stream);

cudaError_t pix2vec_device(long long nside, long long n, const long long* d_pixels, double* d_launch, cudaStream_t stream);

}  // namespace mpf
