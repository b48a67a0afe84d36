// Throughput mode: FP32 gather arithmetic through the per-cell stencil
// records, FP64 RK4 state (with FMA).
#include "mpf_fast.cuh"
#include "mpf_prop_impl.cuh"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <utility>

namespace mpf {
cudaError_t launch_gather_exact(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t stream);

// one instantiation per interpolation order, and per mode (surfaces / sources /
// wide surfaces, per-ray surfaces, direction launches, trajectories)
static void launch_fast_kernel(long long grid, int tpb, const DevTree& T, const DevCosmo& C, const PropParams& P,
                               const double* d_launch, long long n, const PropOut& O, unsigned long long* queue,
                               cudaStream_t stream)
{
    const unsigned g = (unsigned)grid;
    if (P.homogeneous == 2) {
        // Born rays: the field is homogeneous, so the interpolation order does
        // not enter (the Jacobian gathers are TSC)
        if (P.ray_stop) k_propagate_fast<2, true, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
        else k_propagate_fast<2, false, true, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
    } else if (P.ray_stop) {
        if (P.order == 1) k_propagate_fast<1, true, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
        else k_propagate_fast<2, true, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
    } else if (P.wide || P.ray_planes || P.direct || O.traj) {
        if (P.order == 1) k_propagate_fast<1, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
        else k_propagate_fast<2, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
    } else {
        if (P.order == 1) k_propagate_fast<1, false, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
        else k_propagate_fast<2, false, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue);
    }
}

// Launch shape of the persistent kernel.  A batch that fills every SM's
// warp slots runs as blocks of kFastThreads, as many as are resident.  A
// smaller one (the catalogue's last Newton rounds, small ray batches) runs as
// one-warp blocks, one per 32 rays, so that the block scheduler spreads its
// warps over the SMs instead of packing four to an SM: each warp then has an
// SM's FP64 pipe and load slots to itself and its rays finish sooner.
// The kernel's shared-memory layout is sized for kFastThreads and takes any
// smaller block.
static int fast_launch_shape(long long n, int blocks_per_sm, int sms, long long* grid)
{
    const long long warps = (n + 31) / 32;
    const long long slots = (long long)blocks_per_sm * sms * (kFastThreads / 32);
    if (warps < slots) {
        *grid = warps;
        return 32;
    }
    const long long need = (n + kFastThreads - 1) / kFastThreads;
    *grid = std::min<long long>(need, (long long)blocks_per_sm * sms);
    return kFastThreads;
}

// Work-queue counter and occupancy of the persistent kernel, per (device,
// stream): calls on one stream are ordered and may share a counter; calls on
// different streams (or devices) may run at the same time and must not.  One
// 8-byte counter per stream handle seen, kept for the process's lifetime.
// cudaStreamPerThread is one handle value for as many streams as there are
// host threads, so it is keyed per calling thread as well.  The counter is
// zeroed by an asynchronous memset before each launch, so a stream must not
// be shared by host threads that call at the same time (their memsets and
// launches could interleave): each concurrent caller passes its own stream.
struct FastLaunchState {
    unsigned long long* queue = nullptr;
    int blocks_per_sm = 0, sms = 0;
};
static cudaError_t fast_launch_state(cudaStream_t stream, FastLaunchState* out)
{
    static std::mutex mu;
    static std::map<std::tuple<int, cudaStream_t, std::thread::id>, FastLaunchState> states;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const std::thread::id who = (stream == cudaStreamPerThread) ? std::this_thread::get_id() : std::thread::id();
    std::lock_guard<std::mutex> lock(mu);
    FastLaunchState& s = states[std::make_tuple(dev, stream, who)];
    if (!s.queue) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s.blocks_per_sm, k_propagate_fast<2, false, false>, kFastThreads, 0);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaMalloc(&s.queue, sizeof(unsigned long long));
        if (e != cudaSuccess) {
            s = FastLaunchState{};
            return e;
        }
        if (s.blocks_per_sm < 1) s.blocks_per_sm = 1;
    }
    *out = s;
    return cudaSuccess;
}

template <>
cudaError_t launch_propagate<false>(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                                    const PropOut& O, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    // NGP (ORDER = 0) has no interpolation arithmetic to lighten: the float64 kernel
    if (P.order == 0) return launch_propagate<true>(T, C, P, d_launch, n, O, stream);
    FastLaunchState st;
    cudaError_t e = fast_launch_state(stream, &st);
    if (e != cudaSuccess) return e;
    unsigned long long* const queue = st.queue;
    e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    long long grid = 0;
    const int tpb_used = fast_launch_shape(n, st.blocks_per_sm, st.sms, &grid);
    // MPF_STATS=1: count record-path gathers and slow-path fallbacks (diagnostics; serialises the call)
    static const bool want_stats = getenv("MPF_STATS") != nullptr;
    PropOut o2 = O;
    unsigned long long* dstats = nullptr;
    if (want_stats && cudaMalloc(&dstats, ST_N * sizeof(unsigned long long)) == cudaSuccess) {
        cudaMemsetAsync(dstats, 0, ST_N * sizeof(unsigned long long), stream);
        o2.stats = dstats;
    }
    launch_fast_kernel(grid, tpb_used, T, C, P, d_launch, n, o2, queue, stream);
    e = cudaGetLastError();
    if (dstats) {
        unsigned long long h[ST_N];
        cudaMemcpyAsync(h, dstats, sizeof(h), cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        fprintf(stderr, "mpf_stats rk_rec %llu rk_slow %llu post_rec %llu post_slow %llu jac_rec %llu jac_slow %llu cell_changes %llu steps %llu\n",
                h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7]);
#if MPF_DIAG
        unsigned long long dg[4] = {0, 0, 0, 0};
        cudaMemcpyFromSymbol(dg, g_diag, sizeof(dg));
        fprintf(stderr, "mpf_diag restarts %llu full_walks %llu\n", dg[0], dg[1]);
#endif
        cudaFree(dstats);
    }
    return e;
}
cudaError_t launch_gather_fast(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    if (kind == 3) return launch_gather_exact(T, kind, d_xyz, n, d_out, stream);   // NGP: a copy of the cell's record
    k_gather_rec<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(T, kind, d_xyz, n, d_out);
    return cudaGetLastError();
}
}  // namespace mpf

namespace mpf {
// Same launch as launch_propagate<false>, with the work-queue counter supplied
// by the caller (no allocation here).  The counter must be zero on entry.
cudaError_t launch_propagate_fast_with_queue(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch,
                                             long long n, const PropOut& O, unsigned long long* queue, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int tpb = kFastThreads;
    int blocks_per_sm = 0, sms = 0, dev = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_propagate_fast<2, false, false>, tpb, 0);
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    long long grid = 0;
    const int tpb_used = fast_launch_shape(n, blocks_per_sm, sms, &grid);
    launch_fast_kernel(grid, tpb_used, T, C, P, d_launch, n, O, queue, stream);
    return cudaGetLastError();
}
}  // namespace mpf
