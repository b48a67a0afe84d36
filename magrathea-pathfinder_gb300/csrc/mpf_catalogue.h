// Catalogue root-finder driver (mpf_catalogue.cu), called by the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "mpf_device.cuh"
#include "mpf_propagate.cuh"

namespace mpf {

constexpr int kCatalogueFields = 16;

struct CatConst {
    double length, h, mpc, accuracy;
    double vobs[3];
    int max_iterations;
    // jacobiantype = "bundle": Lensing::dbetadtheta from round 5 and at convergence
    int bundle;
    int plane_sachs;      // screen normal: interpolated direction (1) or position (0)
    int stop_bundle;      // StopKind of the bundle rays
    double openingmin;    // radians
    // jacobiantype = "infinitesimal_born": the converged sources' Jacobian
    // along their Born ray (homogeneous field on the octree's levels)
    int born;
};

struct CatRotation {
    double m[3][3];
};

struct CatRunStats {
    long long rays;
    long long photon_steps;
    long long photon_steps_jacobian;
    int iterations;
    int launches;
};

// d_src: n rows of `stride` doubles on the device; d_rows: n x 16 on the
// device.  Synchronises `stream` once per Newton round (the size of the next
// round decides its launch).  h_status: the propagate status bits.
cudaError_t catalogue_newton(const DevTree& T, const DevCosmo& C, const CatConst& K, const CatRotation* rot, bool exact,
                             int order, unsigned nsteps, long long n, const double* d_src, int stride, double* d_rows,
                             CatRunStats* stats, unsigned* h_status, cudaStream_t stream);

}  // namespace mpf
