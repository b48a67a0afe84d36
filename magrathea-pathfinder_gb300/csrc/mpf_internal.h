// Internal host-side structures shared by the CUDA translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mpf_gb300.h"
#include "mpf_device.cuh"
#include "mpf_propagate.cuh"

struct mpf_octree {
    int device;
    int64_t n;
    int64_t nnodes;
    int level_min, level_max;
    mpf::DevTree tree;       // device pointers inside
    ulonglong2* keys;
    float4* grad;
    float4* scal;
    int2* node;
    int* grid;
    int4* stencil;
    float4* vel;             // velocity field (vx, vy, vz, 0) per cell, or null
    int64_t deposit_pairs;   // (cell, particle, vertex) pairs of the last velocity deposit
};

struct mpf_cosmology {
    int device;
    int n;
    double* t;
    double* a;
    double* dadt;
    double* d2adt2;
    int* lut;
    int nlut;
    double t0, lut_scale;
    double* slope_a;
    double* slope_dadt;
    float2* seg;
};

// device view of a cosmology table
inline mpf::DevCosmo dev_cosmo(const mpf_cosmology* c)
{
    return mpf::DevCosmo{c->t, c->a, c->dadt, c->n, c->lut, c->nlut, c->t0, c->lut_scale, c->slope_a, c->slope_dadt, c->seg};
}

// sets the calling thread's mpf_last_error() message; returns code
int mpf_internal_set_error(int code, const char* msg);

// checks an mpf_params block and fills the device parameters (false: bad input)
bool mpf_internal_fill_params(const mpf_params* p, mpf::PropParams& P);

namespace mpf {

// exclusive scan of n int32 values in place on `stream`; returns the total
int64_t exclusive_scan(int* d, int64_t n, cudaStream_t stream);

template <bool EXACT>
cudaError_t launch_propagate(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                             const PropOut& O, cudaStream_t stream);

cudaError_t launch_gather(const DevTree& T, int kind, bool exact, const double* d_xyz, long long n, void* d_out,
                          cudaStream_t stream);

// Autotuned launch shapes (mpf_prop_fast.cu, mpf_cat_persist.cu): false until
// tuned.  rates: photon-steps/s of the candidates (4 for the propagate kernel:
// 128 x 1, 64 x 1, 32 x 1, 128 x 2 threads x claim depth; 3 for the
// catalogue: 128, 64, 32 threads).
bool tuned_shape(int dev, const DevTree& T, int mode, int* tpb, int* depth, double* rates);
int plain_fast_mode(int order, bool velocity);
bool catalogue_tuned_shape(int dev, const DevTree& T, int order, int* tpb, double* rates);
// forget an octree's tuned shapes when its arrays are freed
void forget_tuned_shape(const void* keys);
void catalogue_forget_tuned_shape(const void* keys);

}  // namespace mpf
