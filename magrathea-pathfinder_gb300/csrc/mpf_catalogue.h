// Catalogue root-finder driver (mpf_catalogue.cu), called by the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "mpf_device.cuh"
#include "mpf_propagate.cuh"

namespace mpf {

constexpr int kCatalogueFields = 16;

// status bit of a catalogue call whose device work queue lost a source
constexpr unsigned kCatQueueError = 1u << 8;

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

// Whether the persistent work-queue driver serves these parameters (the
// FP32-gather kernel with the infinitesimal Jacobian).
bool catalogue_persistent_applies(const CatConst& K, bool exact, int order);

// The persistent driver (mpf_cat_persist.cu): one CUDA graph launch per call,
// one synchronisation at its end.  queue_error: the work queue lost a source
// (a bounded wait ran out); catalogue_queue_message() then describes it.
cudaError_t catalogue_newton_persistent(const DevTree& T, const DevCosmo& C, const CatConst& K, const CatRotation* rot,
                                        int order, unsigned nsteps, long long n, const double* d_src, int stride,
                                        double* d_rows, CatRunStats* stats, unsigned* h_status, bool* queue_error,
                                        cudaStream_t stream);
const char* catalogue_queue_message();

// d_src: n rows of `stride` doubles on the device; d_rows: n x 16 on the
// device.  The FP32-gather kernel with the infinitesimal Jacobian runs the
// persistent driver; otherwise the call synchronises `stream` once per Newton
// round (the size of the next round decides its launch).  h_status: the
// propagate status bits, and kCatQueueError.
cudaError_t catalogue_newton(const DevTree& T, const DevCosmo& C, const CatConst& K, const CatRotation* rot, bool exact,
                             int order, unsigned nsteps, long long n, const double* d_src, int stride, double* d_rows,
                             CatRunStats* stats, unsigned* h_status, cudaStream_t stream);

}  // namespace mpf
