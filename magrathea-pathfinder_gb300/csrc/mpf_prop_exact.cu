// Reference-order (bit-exact) mode.  Must be compiled with -fmad=false.
#include "mpf_prop_impl.cuh"

namespace mpf {
template <>
cudaError_t launch_propagate<true>(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                                   const PropOut& O, cudaStream_t stream)
{
    return launch_propagate_impl<true>(T, C, P, d_launch, n, O, stream);
}
cudaError_t launch_gather_exact(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t stream)
{
    return launch_gather_impl<true>(T, kind, d_xyz, n, d_out, stream);
}
}  // namespace mpf
