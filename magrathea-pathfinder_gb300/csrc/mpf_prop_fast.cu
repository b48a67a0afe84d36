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

// The kernel instantiation a launch uses: per interpolation order and mode
// (surfaces / sources / wide surfaces, per-ray surfaces, direction launches,
// trajectories; Born rays; a velocity-field octree, plain surfaces only).
static int fast_mode(const DevTree& T, const PropParams& P, const PropOut& O)
{
    if (P.homogeneous == 2) return P.ray_stop ? 0 : 1;
    if (P.ray_stop) return (P.order == 1) ? 2 : 3;
    if (P.wide || P.ray_planes || P.direct || O.traj) return (P.order == 1) ? 4 : 5;
    if (T.vel) return (P.order == 1) ? 8 : 9;
    return (P.order == 1) ? 6 : 7;
}

// A velocity-field octree runs the FP32-gather kernel in the plain mode only
// (surface records: propagation and maps); its other modes (Born, source,
// bundle and trajectory rays) run the float64 kernel.
static bool fast_mode_supported(const DevTree& T, const PropParams& P, const PropOut& O)
{
    const int m = fast_mode(T, P, O);
    return !T.vel || m == 8 || m == 9;
}

// Launches rays [lo, n) of the batch as grid blocks of tpb threads, each warp
// claiming 32 x depth rays at a time.
static void launch_fast_kernel(long long grid, int tpb, int depth, long long lo, const DevTree& T, const DevCosmo& C,
                               const PropParams& P, const double* d_launch, long long n, const PropOut& O,
                               unsigned long long* queue, cudaStream_t stream)
{
    const unsigned g = (unsigned)grid;
    switch (fast_mode(T, P, O)) {
    // Born rays: the field is homogeneous, so the interpolation order does
    // not enter (the Jacobian gathers are TSC)
    case 0: k_propagate_fast<2, true, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 1: k_propagate_fast<2, false, true, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 2: k_propagate_fast<1, true, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 3: k_propagate_fast<2, true, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 4: k_propagate_fast<1, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 5: k_propagate_fast<2, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 6: k_propagate_fast<1, false, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 8: k_propagate_fast<1, false, false, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    case 9: k_propagate_fast<2, false, false, false, true><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
    default: k_propagate_fast<2, false, false><<<g, tpb, 0, stream>>>(T, C, P, d_launch, n, O, queue, depth, lo); break;
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

// ---------------------------------------------------------------------------
// Autotuner of the persistent launch shape: threads per block and the depth
// of a warp's claim on the work queue (32 x depth rays).  The first batch of
// at least kTuneMinRays rays for a (device, octree, kernel mode) is split into
// one slice per candidate shape; each slice is traced with its shape and
// timed with CUDA events, and its photon-steps are summed on the device.  The
// shape with the most photon-steps per second is kept for that key and used
// by every later launch.  Every ray is traced exactly once and its results do
// not depend on the shape, so tuning changes no output; the tuning call
// waits for its slices.  MPF_AUTOTUNE=0 keeps the default shape.
struct TuneShape {
    int tpb, depth;
};
static const TuneShape kTuneCandidates[] = {{kFastThreads, 1}, {64, 1}, {32, 1}, {kFastThreads, 2}};
constexpr int kTuneN = 4;
constexpr long long kTuneMinRays = 1ll << 17;

struct TuneResult {
    int done = 0;
    TuneShape best{kFastThreads, 1};
    double rate[kTuneN] = {0, 0, 0, 0};   // photon-steps/s of each candidate
};
static std::mutex g_tune_mu;
static std::map<std::tuple<int, const void*, int>, TuneResult> g_tune;

static __global__ void k_sum_steps(const long long* __restrict__ steps, long long lo, long long hi,
                                   unsigned long long* __restrict__ out)
{
    unsigned long long s = 0;
    for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (long long)gridDim.x * blockDim.x)
        s += (unsigned long long)(steps[i] > 0 ? steps[i] - 1 : 0);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// resident blocks per SM of the kernel at tpb threads (at least 1)
static int blocks_per_sm_at(int tpb)
{
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_propagate_fast<2, false, false>, tpb, 0) != cudaSuccess) b = 1;
    return std::max(1, b);
}

// the grid of a shape for `rays` rays: every SM's resident blocks, fewer when
// the rays do not fill them
static long long shape_grid(const TuneShape& sh, long long rays, int sms)
{
    const long long need = (rays + (long long)sh.tpb * sh.depth - 1) / ((long long)sh.tpb * sh.depth);
    return std::max<long long>(1, std::min<long long>(need, (long long)blocks_per_sm_at(sh.tpb) * sms));
}

// Tunes the shape on this batch (tracing all of it); fills *res.
static cudaError_t tune_and_launch(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch,
                                   long long n, const PropOut& O, unsigned long long* queue, int sms, cudaStream_t stream,
                                   TuneResult* res)
{
    unsigned long long* dsum = nullptr;
    cudaEvent_t ev[kTuneN + 1] = {};
    cudaError_t e = cudaMalloc(&dsum, kTuneN * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(dsum, 0, kTuneN * sizeof(unsigned long long), stream);
    for (int k = 0; k <= kTuneN && e == cudaSuccess; ++k) e = cudaEventCreate(&ev[k]);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], stream);
    const long long slice = n / kTuneN;
    for (int k = 0; k < kTuneN && e == cudaSuccess; ++k) {
        const long long lo = k * slice, hi = (k == kTuneN - 1) ? n : lo + slice;
        const TuneShape& sh = kTuneCandidates[k];
        e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), stream);
        if (e != cudaSuccess) break;
        launch_fast_kernel(shape_grid(sh, hi - lo, sms), sh.tpb, sh.depth, lo, T, C, P, d_launch, hi, O, queue, stream);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        e = cudaEventRecord(ev[k + 1], stream);
        if (e == cudaSuccess) k_sum_steps<<<64, 256, 0, stream>>>(O.steps, lo, hi, dsum + k);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    unsigned long long ps[kTuneN] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(ps, dsum, sizeof(ps), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) {
        double best = -1.0;
        for (int k = 0; k < kTuneN; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            res->rate[k] = (ms > 0.f) ? (double)ps[k] / (ms * 1e-3) : 0.0;
            if (res->rate[k] > best) {
                best = res->rate[k];
                res->best = kTuneCandidates[k];
            }
        }
        res->done = 1;
    }
    for (int k = 0; k <= kTuneN; ++k)
        if (ev[k]) cudaEventDestroy(ev[k]);
    if (dsum) cudaFree(dsum);
    return e;
}

// the tuned shape of (device, octree, kernel mode), or false
bool tuned_shape(int dev, const DevTree& T, int mode, int* tpb, int* depth, double* rates)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(std::make_tuple(dev, (const void*)T.keys, mode));
    if (it == g_tune.end() || !it->second.done) return false;
    *tpb = it->second.best.tpb;
    *depth = it->second.best.depth;
    if (rates)
        for (int k = 0; k < kTuneN; ++k) rates[k] = it->second.rate[k];
    return true;
}

// drops the tuned shapes of an octree whose device arrays are freed (a later
// octree may reuse the addresses)
void forget_tuned_shape(const void* keys)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (auto it = g_tune.begin(); it != g_tune.end();) {
        if (std::get<1>(it->first) == keys) it = g_tune.erase(it);
        else ++it;
    }
}

// the kernel mode of the plain (surface-record) instantiation for `order`
// (8 / 9 on a velocity-field octree)
int plain_fast_mode(int order, bool velocity) { return velocity ? ((order == 1) ? 8 : 9) : ((order == 1) ? 6 : 7); }

template <>
cudaError_t launch_propagate<false>(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch, long long n,
                                    const PropOut& O, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    // NGP (ORDER = 0) has no interpolation arithmetic to lighten: the float64 kernel
    if (P.order == 0 || !fast_mode_supported(T, P, O)) return launch_propagate<true>(T, C, P, d_launch, n, O, stream);
    FastLaunchState st;
    cudaError_t e = fast_launch_state(stream, &st);
    if (e != cudaSuccess) return e;
    unsigned long long* const queue = st.queue;
    e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    long long grid = 0;
    int tpb_used = fast_launch_shape(n, st.blocks_per_sm, st.sms, &grid);
    int depth = 1;
    // MPF_STATS=1: count record-path gathers and slow-path fallbacks (diagnostics; serialises the call)
    static const bool want_stats = getenv("MPF_STATS") != nullptr;
    static const bool want_tune = !(getenv("MPF_AUTOTUNE") && getenv("MPF_AUTOTUNE")[0] == '0');
    if (tpb_used == kFastThreads && want_tune && !want_stats) {
        // a batch that fills the GPU: the tuned shape of this octree and kernel mode
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        const auto key = std::make_tuple(dev, (const void*)T.keys, fast_mode(T, P, O));
        TuneResult res;
        bool have = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            auto it = g_tune.find(key);
            if (it != g_tune.end() && it->second.done) {
                res = it->second;
                have = true;
            }
        }
        if (!have && n >= kTuneMinRays) {
            e = tune_and_launch(T, C, P, d_launch, n, O, queue, st.sms, stream, &res);
            if (e == cudaSuccess) {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                g_tune[key] = res;
            }
            return e;
        }
        if (have) {
            tpb_used = res.best.tpb;
            depth = res.best.depth;
            grid = shape_grid(res.best, n, st.sms);
        }
    }
    PropOut o2 = O;
    unsigned long long* dstats = nullptr;
    if (want_stats && cudaMalloc(&dstats, ST_N * sizeof(unsigned long long)) == cudaSuccess) {
        cudaMemsetAsync(dstats, 0, ST_N * sizeof(unsigned long long), stream);
        o2.stats = dstats;
    }
    launch_fast_kernel(grid, tpb_used, depth, 0, T, C, P, d_launch, n, o2, queue, stream);
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
    launch_fast_kernel(grid, tpb_used, 1, 0, T, C, P, d_launch, n, O, queue, stream);
    return cudaGetLastError();
}
}  // namespace mpf
