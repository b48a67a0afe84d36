// Kernel launchers for one arithmetic mode; included once by
// mpf_prop_exact.cu (built with -fmad=false: the reference's float64
// operation order and rounding, bit-exact gathers and trajectories) and once
// by mpf_prop_fast.cu (FP32 gather arithmetic, FP64 state with FMA).
#pragma once
#include "mpf_internal.h"

namespace mpf {

template <bool EXACT>
__global__ void k_gather(DevTree T, int kind, const double* __restrict__ xyz, long long n, void* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (kind == 0) {
        ((long long*)out)[i] = locate(T, x, y, z).cell;
        return;
    }
    // kind 1: CIC, 2: TSC, 3: NGP
    const Field7 f = (kind == 1) ? cic<EXACT>(T, x, y, z, true) : (kind == 3) ? ngp(T, x, y, z) : tsc<EXACT>(T, x, y, z, true);
    float* o = (float*)out + 7 * i;
    o[0] = f.rho; o[1] = f.phi; o[2] = f.dx; o[3] = f.dy; o[4] = f.dz; o[5] = f.a; o[6] = f.dt;
}

template <bool EXACT>
cudaError_t launch_propagate_impl(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                                  const PropOut& O, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int tpb = 128;
    const unsigned grid = (unsigned)((n + tpb - 1) / tpb);
    if (P.ray_stop) k_propagate<EXACT, true><<<grid, tpb, 0, stream>>>(T, C, P, d_launch, n, O);
    else k_propagate<EXACT, false><<<grid, tpb, 0, stream>>>(T, C, P, d_launch, n, O);
    return cudaGetLastError();
}

template <bool EXACT>
cudaError_t launch_gather_impl(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int tpb = 128;
    k_gather<EXACT><<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, stream>>>(T, kind, d_xyz, n, d_out);
    return cudaGetLastError();
}

}  // namespace mpf
