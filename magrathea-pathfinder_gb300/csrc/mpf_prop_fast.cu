// Throughput mode: FP32 gather arithmetic through the per-ray cell window,
// FP64 RK4 state (with FMA).
#include "mpf_fast.cuh"
#include "mpf_prop_impl.cuh"

#include <algorithm>

namespace mpf {
template <>
cudaError_t launch_propagate<false>(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                                    const PropOut& O, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int tpb = kFastThreads;
    const size_t smem = (size_t)kWin3 * tpb * sizeof(int);
    static int blocks_per_sm = 0, sms = 0;
    static unsigned long long* queue = nullptr;   // one work counter per process (calls on a stream are ordered)
    if (blocks_per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute(k_propagate_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_propagate_fast, tpb, smem);
        int dev = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaMalloc(&queue, sizeof(unsigned long long));
        if (e != cudaSuccess) { blocks_per_sm = 0; return e; }
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    const long long need = (n + tpb - 1) / tpb;
    const long long grid = std::min<long long>(need, (long long)blocks_per_sm * sms);
    k_propagate_fast<<<(unsigned)grid, tpb, smem, stream>>>(T, C, P, d_launch, n, O, queue);
    return cudaGetLastError();
}
cudaError_t launch_gather_fast(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t stream)
{
    return launch_gather_impl<false>(T, kind, d_xyz, n, d_out, stream);
}
}  // namespace mpf
