// Catalogue root-finder as one persistent launch fed by a device work queue
// (fast mode, jacobiantype = "infinitesimal"): Catalogues::iterateNewtonMethod
// and newtonMethod2d (src/catalogues.h:410-783) for a whole batch of sources.
//
// The queue holds work items, one per source that needs a ray: the source's
// index and whether the ray is a Newton ray or the re-trace that gives a
// converged source its lensing Jacobian.  Each warp of the persistent kernel
// claims up to 32 items, traces their rays (the propagate kernel's source
// mode: stop at the source radius, one record at the crossing), applies the
// Newton update to each source, and pushes the sources that need another ray
// back on the queue.  Sources advance at their own pace: there are no rounds,
// no host synchronisation between rays, and no round that waits for its
// slowest ray while the SMs idle.
//
// The call is one CUDA graph: the sources' set-up and their sort by radius
// bin and direction (so that a warp's 32 rays are neighbours of about the
// same length), the queue's initial fill and the persistent kernel.  The
// graph, its scratch buffers and a device block of the call's arguments form
// a plan, kept per (device, stream, interpolation order) and reused by every
// later call with at most as many sources: a call writes its arguments into
// the block, points the persistent kernel at its octree, cosmology and
// parameters, and launches the graph.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "mpf_fast.cuh"
#include "mpf_internal.h"
#include "mpf_cat_device.cuh"

namespace mpf {

// The call's arguments, read by the graph's kernels from device memory.
struct CatCall {
    const double* src;
    double* rows;
    long long n;
    int stride;
    int has_rot;
    CatRotation rot;
};

// Queue control words.  kQFault*: where the first queue fault happened (for a
// producer, the position, the slot's word and head / tail at that moment; for
// a consumer, the position and tail), reported with the error.
enum { kQHead = 0, kQTail, kQFlight, kQRays, kQIter, kQFault0, kQFault1, kQFault2, kQFault3, kQFault4, kQFault5, kQWords };
// queue status bits (counter 1): a bounded wait on a slot ran out
constexpr unsigned kQueueSlotTimeout = 1u;   // a consumer's item was not written within kSlotNs
constexpr unsigned kQueueSlotBusy = 2u;      // a producer's slot was not freed within kSlotNs

// A ring slot is one 64-bit word: the slot's turn in the high half, the item
// in the low half.  Position p of the queue uses slot p % cap in lap
// L = p / cap: its producer waits for turn 2L (the slot free for lap L) and
// writes the item with turn 2L + 1; its consumer waits for turn 2L + 1, takes
// the item and leaves turn 2L + 2 (free for lap L + 1).  A warp can be delayed
// for any time between claiming a position and reading it, so the turn, not
// the distance between head and tail, keeps a late reader's item from being
// overwritten by the next lap.
__host__ __device__ __forceinline__ unsigned long long slot_word(unsigned long long turn, int item)
{
    return (turn << 32) | (unsigned long long)(unsigned)item;
}

// A plan's device buffers (fixed for the plan's life).
struct CatPlanDev {
    const CatCall* call;
    CatState* state;
    uint32_t *key0, *key1;
    int *val0, *val1;
    int* hist;                  // 16 x ntiles digit counts of the sort
    long long ntiles;           // sort tiles of kPSortTile sources for the capacity
    unsigned long long* items;  // the queue's ring of `cap` slots (turn, item)
    long long cap;
    unsigned long long* ctl;    // kQWords control words
    unsigned* cnt;              // [0] sources with a direction, [1] queue status bits
    unsigned long long* psteps; // [0] accepted steps, [1] those traced with the Jacobian
    double* radius;             // per source: the stop radius of its rays
    double* rec;                // per source: its last ray's record (kSourceFields)
    long long* steps;           // per source: its last ray's trajectory size
    unsigned* status;           // propagate status bits
};

constexpr int kPSortTile = 256;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void k_p_reset(CatPlanDev D)
{
    if (threadIdx.x < kQWords) D.ctl[threadIdx.x] = 0ull;
    if (threadIdx.x < 2) {
        D.cnt[threadIdx.x] = 0u;
        D.psteps[threadIdx.x] = 0ull;
    }
    if (threadIdx.x == 0) *D.status = 0u;
}

__global__ void k_p_init(CatPlanDev D)
{
    const CatCall& A = *D.call;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    cat_init_one(i, A.src, A.stride, A.rot, A.has_rot, D.state, A.rows, D.key0, D.val0, D.cnt);
    D.radius[i] = D.state[i].dist;
}

// Stable LSD radix sort pass over the call's n sources (4-bit digit at `shift`):
// per-tile digit counts, one-block exclusive scan, scatter.
__global__ void k_p_hist(CatPlanDev D, const uint32_t* __restrict__ key, int shift)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= D.ntiles) return;
    int h[16];
    for (int d = 0; d < 16; ++d) h[d] = 0;
    const long long e = min(D.call->n, (t + 1) * kPSortTile);
    for (long long i = t * kPSortTile; i < e; ++i) ++h[(key[i] >> shift) & 15u];
    for (int d = 0; d < 16; ++d) D.hist[d * D.ntiles + t] = h[d];
}

// Exclusive prefix sum of len ints in place, one block of 1024 threads: each
// thread scans a contiguous chunk, the chunk totals are scanned in shared
// memory, then each chunk is offset.  No host synchronisation.
__global__ void __launch_bounds__(1024) k_p_scan(int* __restrict__ d, long long len)
{
    __shared__ long long part[1024];
    const int tid = threadIdx.x;
    const long long chunk = (len + 1023) / 1024;
    const long long b = min(len, tid * chunk), e = min(len, b + chunk);
    long long s = 0;
    for (long long i = b; i < e; ++i) s += d[i];
    part[tid] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const long long v = (tid >= off) ? part[tid - off] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    long long run = part[tid] - s;   // exclusive offset of this chunk
    for (long long i = b; i < e; ++i) {
        const int v = d[i];
        d[i] = (int)run;
        run += v;
    }
}

__global__ void k_p_scatter(CatPlanDev D, const uint32_t* __restrict__ key, const int* __restrict__ val, int shift,
                            uint32_t* __restrict__ key2, int* __restrict__ val2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= D.ntiles) return;
    int o[16];
    for (int d = 0; d < 16; ++d) o[d] = D.hist[d * D.ntiles + t];
    const long long e = min(D.call->n, (t + 1) * kPSortTile);
    for (long long i = t * kPSortTile; i < e; ++i) {
        const uint32_t k = key[i];
        const int j = o[(k >> shift) & 15u]++;
        key2[j] = k;
        val2[j] = val[i];
    }
}

// The queue's first content: every source with a direction, in sort order,
// for its first Newton ray.
__global__ void k_p_fill(CatPlanDev D)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long m = (long long)D.cnt[0];
    // lap 0: the first m positions written (turn 1), the rest free (turn 0)
    if (j < D.cap) D.items[j] = (j < m) ? slot_word(1ull, D.val0[j] << 1) : slot_word(0ull, -1);
    if (j == 0) D.ctl[kQTail] = (unsigned long long)m;
}

// The persistent root-finder.  Waits are bounded: an idle warp (empty queue,
// work still in flight elsewhere) sleeps and gives up after kIdleNs (the warps
// holding work push and claim their own continuations, so nothing is lost);
// a consumer waits for its item and a producer for its slot's previous reader
// at most kSlotNs, after which the kernel records a queue fault for the host
// and the lane leaves the item.
constexpr unsigned long long kIdleNs = 30ull * 1000000000ull;
constexpr unsigned long long kSlotNs = 2ull * 1000000000ull;

template <int ORDER>
__global__ void MPF_FAST_BOUNDS k_cat_persistent(DevTree T, DevCosmo C, CatPlanDev D, PropParams P, CatConst K)
{
    __shared__ double jac_sums[6 * kFastThreads];
    __shared__ float jac_terms[12 * kFastThreads];
    const JacSums J{jac_sums + threadIdx.x, jac_terms + threadIdx.x};
    const int lane = threadIdx.x & 31;
    const PropOut O{D.steps, nullptr, D.rec, D.status, nullptr};
    unsigned long long* const ctl = D.ctl;
    const unsigned long long cap = (unsigned long long)D.cap;
    for (;;) {
        unsigned long long base = 0;
        int cnt = 0;
        if (lane == 0) {
            const unsigned long long t0 = global_ns();
            for (;;) {
                // in flight first: a source is pushed before its ray leaves the count
                const unsigned long long fl = atomicAdd(ctl + kQFlight, 0ull);
                const unsigned long long h = atomicAdd(ctl + kQHead, 0ull);
                const unsigned long long t = atomicAdd(ctl + kQTail, 0ull);
                if (h < t) {
                    const unsigned long long c = min(32ull, t - h);
                    atomicAdd(ctl + kQFlight, c);
                    if (atomicCAS(ctl + kQHead, h, h + c) == h) {
                        base = h;
                        cnt = (int)c;
                        break;
                    }
                    atomicAdd(ctl + kQFlight, (unsigned long long)(-(long long)c));
                    continue;
                }
                if (fl == 0ull) break;                       // nothing queued, nothing in flight: done
                if (global_ns() - t0 > kIdleNs) break;
                __nanosleep(2000);
            }
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        cnt = __shfl_sync(0xffffffffu, cnt, 0);
        if (cnt == 0) break;
        int item = -1;
        if (lane < cnt) {
            const unsigned long long pos = base + (unsigned long long)lane;
            const unsigned long long lap = pos / cap;
            unsigned long long* const sw = D.items + (long long)(pos % cap);
            const unsigned long long t0 = global_ns();
            for (;;) {
                const unsigned long long v = atomicAdd(sw, 0ull);
                if ((v >> 32) == 2ull * lap + 1ull) {
                    item = (int)(unsigned)(v & 0xffffffffull);
                    atomicExch(sw, slot_word(2ull * lap + 2ull, -1));
                    break;
                }
                if (global_ns() - t0 > kSlotNs) {
                    atomicOr(D.cnt + 1, kQueueSlotTimeout);
                    if (atomicCAS(ctl + kQFault4, 0ull, pos + 1) == 0ull) ctl[kQFault5] = atomicAdd(ctl + kQTail, 0ull);
                    break;
                }
                __nanosleep(64);
            }
        }
        int push = -1;
        if (item >= 0) {
            const int s = item >> 1;
            const bool retrace = (item & 1) != 0;
            const CatState& S = D.state[s];
            const int it = S.it;
            // launch toward (phi, theta) from the observer (integrator.h:305-329)
            const double st = sin(S.theta);
            const double L[6] = {0.0, 0.0, 0.0, cos(S.phi) * st, sin(S.phi) * st, cos(S.theta)};
            // rounds 0-1 (identity Newton matrix) trace without the lensing
            // Jacobian; from round 2 on, and for the re-trace, with it
            PropParams Pl = P;
            Pl.jacobian = (retrace || it >= 2) ? 1 : 0;
            propagate_fast<ORDER, true, false>(T, C, Pl, L, s, O, J);
            const double* o = D.rec + (long long)kSourceFields * s;
            if (retrace) {
                cat_final_jacobian(D.call->rows + (long long)kCatalogueFields * s, o, D.steps[s], D.psteps, 0);
            } else {
                const int r = cat_update(s, it, Pl.jacobian, K, D.state, D.call->rows, D.steps[s], o, D.psteps);
                atomicMax(ctl + kQIter, (unsigned long long)(it + 1));
                if (r == kCatContinue) {
                    D.state[s].it = it + 1;
                    push = s << 1;
                } else if (r == kCatRetrace) {
                    push = (s << 1) | 1;
                }
            }
        }
        // warp-aggregated push of the sources that need another ray
        const unsigned want = __ballot_sync(0xffffffffu, push >= 0);
        if (want) {
            unsigned long long pb = 0;
            if (lane == 0) pb = atomicAdd(ctl + kQTail, (unsigned long long)__popc(want));
            pb = __shfl_sync(0xffffffffu, pb, 0);
            if (push >= 0) {
                const unsigned long long pos = pb + (unsigned long long)__popc(want & ((1u << lane) - 1u));
                const unsigned long long lap = pos / cap;
                unsigned long long* const sw = D.items + (long long)(pos % cap);
                const unsigned long long t0 = global_ns();
                for (;;) {
                    // the slot is free for this lap once the previous lap's reader took its item
                    if ((atomicAdd(sw, 0ull) >> 32) == 2ull * lap) {
                        atomicExch(sw, slot_word(2ull * lap + 1ull, push));
                        break;
                    }
                    if (global_ns() - t0 > kSlotNs) {
                        atomicOr(D.cnt + 1, kQueueSlotBusy);
                        if (atomicCAS(ctl + kQFault0, 0ull, pos + 1) == 0ull) {
                            ctl[kQFault1] = atomicAdd(sw, 0ull);
                            ctl[kQFault2] = atomicAdd(ctl + kQHead, 0ull);
                            ctl[kQFault3] = atomicAdd(ctl + kQTail, 0ull);
                        }
                        break;
                    }
                    __nanosleep(64);
                }
            }
        }
        const unsigned traced = __ballot_sync(0xffffffffu, item >= 0);
        __threadfence();
        __syncwarp();
        if (lane == 0) {
            atomicAdd(ctl + kQRays, (unsigned long long)__popc(traced));
            atomicAdd(ctl + kQFlight, (unsigned long long)(-(long long)cnt));
        }
    }
}

namespace {

unsigned nblocks(long long n, int tpb) { return (unsigned)std::max<long long>(1, (n + tpb - 1) / tpb); }

struct CatPlan {
    int device = 0;
    int order = 2;
    long long cap = 0;
    CatPlanDev D{};
    CatCall* d_call = nullptr;
    std::vector<void*> bufs;
    cudaGraph_t graph = nullptr;       // kept: the exec's node updates refer to its nodes
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t pnode = nullptr;   // the persistent kernel's node
    cudaKernelNodeParams pparams{};
    int grid = 0, tpb = 0;
    int kernels = 0;                   // kernel nodes of the graph

    ~CatPlan()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void* b : bufs) cudaFree(b);
    }
};

template <class X>
cudaError_t dalloc(CatPlan& pl, X** p, size_t count)
{
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(X));
    if (e == cudaSuccess) {
        pl.bufs.push_back(q);
        *p = (X*)q;
    }
    return e;
}

// Scratch, launch shape and graph of a plan for up to `cap` sources.  P: the
// source-mode propagation parameters (its stop radii are the plan's own).
cudaError_t plan_build(CatPlan& pl, const DevTree& T, const DevCosmo& C, PropParams P, const CatConst& K)
{
    cudaError_t e = cudaGetDevice(&pl.device);
    const long long cap = pl.cap;
    CatPlanDev& D = pl.D;
    // one slot per source plus spare slots: a push rarely waits for a reader
    D.cap = cap + 1024;
    D.ntiles = (cap + kPSortTile - 1) / kPSortTile;
    if (e == cudaSuccess) e = dalloc(pl, &pl.d_call, 1);
    if (e == cudaSuccess) e = dalloc(pl, &D.state, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.key0, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.key1, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.val0, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.val1, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.hist, (size_t)(16 * D.ntiles));
    if (e == cudaSuccess) e = dalloc(pl, &D.items, (size_t)D.cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.ctl, (size_t)kQWords);
    if (e == cudaSuccess) e = dalloc(pl, &D.cnt, 2);
    if (e == cudaSuccess) e = dalloc(pl, &D.psteps, 2);
    if (e == cudaSuccess) e = dalloc(pl, &D.radius, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.rec, (size_t)cap * kSourceFields);
    if (e == cudaSuccess) e = dalloc(pl, &D.steps, (size_t)cap);
    if (e == cudaSuccess) e = dalloc(pl, &D.status, 1);
    if (e != cudaSuccess) return e;
    D.call = pl.d_call;
    P.ray_stop = D.radius;
    // persistent grid: every SM's resident blocks of the propagate launch bounds
    int bps = 0, sms = 0;
    e = (pl.order == 1) ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_cat_persistent<1>, kFastThreads, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_cat_persistent<2>, kFastThreads, 0);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pl.device);
    if (e != cudaSuccess) return e;
    pl.tpb = kFastThreads;
    pl.grid = std::max(1, bps) * sms;
    // the set-up is captured on a stream of its own (the legacy default
    // stream cannot capture); the graph then launches on any stream
    cudaStream_t cs = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return e;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const int tpb = 256;
        k_p_reset<<<1, 32, 0, cs>>>(D);
        k_p_init<<<nblocks(cap, tpb), tpb, 0, cs>>>(D);
        uint32_t *ka = D.key0, *kb = D.key1;
        int *va = D.val0, *vb = D.val1;
        for (int shift = 0; shift < 32; shift += 4) {
            k_p_hist<<<nblocks(D.ntiles, tpb), tpb, 0, cs>>>(D, ka, shift);
            k_p_scan<<<1, 1024, 0, cs>>>(D.hist, 16 * D.ntiles);
            k_p_scatter<<<nblocks(D.ntiles, tpb), tpb, 0, cs>>>(D, ka, va, shift, kb, vb);
            std::swap(ka, kb);
            std::swap(va, vb);
        }
        k_p_fill<<<nblocks(D.cap, tpb), tpb, 0, cs>>>(D);
        e = cudaGetLastError();
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess) e = e2;
    }
    cudaStreamDestroy(cs);
    // the persistent kernel is a node of its own after the captured set-up,
    // so that each call can point it at its octree, cosmology and parameters;
    // it depends on the set-up's last nodes (the nodes no edge leaves)
    std::vector<cudaGraphNode_t> deps;
    if (e == cudaSuccess) {
        size_t nn = 0, ne = 0;
        e = cudaGraphGetNodes(g, nullptr, &nn);
        if (e == cudaSuccess) e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne);
        std::vector<cudaGraphNode_t> nodes(nn), from(ne), to(ne);
        if (e == cudaSuccess) e = cudaGraphGetNodes(g, nodes.data(), &nn);
        if (e == cudaSuccess && ne > 0) e = cudaGraphGetEdges(g, from.data(), to.data(), nullptr, &ne);
        for (cudaGraphNode_t nd : nodes)
            if (std::find(from.begin(), from.end(), nd) == from.end()) deps.push_back(nd);
        if (e == cudaSuccess && deps.empty()) e = cudaErrorInvalidValue;
    }
    if (e == cudaSuccess) {
        void* args[5] = {(void*)&T, (void*)&C, (void*)&D, (void*)&P, (void*)&K};
        cudaKernelNodeParams kp{};
        kp.func = (pl.order == 1) ? (void*)k_cat_persistent<1> : (void*)k_cat_persistent<2>;
        kp.gridDim = dim3((unsigned)pl.grid);
        kp.blockDim = dim3((unsigned)pl.tpb);
        kp.sharedMemBytes = 0;
        kp.kernelParams = args;
        kp.extra = nullptr;
        e = cudaGraphAddKernelNode(&pl.pnode, g, deps.data(), deps.size(), &kp);
        size_t nn = 0;
        if (e == cudaSuccess) e = cudaGraphGetNodes(g, nullptr, &nn);
        pl.kernels = (int)nn;
        pl.pparams = kp;
        pl.pparams.kernelParams = nullptr;
    }
    pl.graph = g;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&pl.exec, g, 0);
    return e;
}

// Autotuning of the persistent kernel's block size (the grid is every SM's
// resident blocks at that size): the first kCatTuneN calls of at least
// kCatTuneMin sources on a (device, octree, order) run one candidate each and
// are timed (a call waits for its result anyway); later calls use the fastest
// in photon-steps per second.  A source's rows do not depend on the block
// size.  MPF_AUTOTUNE=0 keeps kFastThreads.
constexpr int kCatTuneN = 3;
constexpr long long kCatTuneMin = 1ll << 16;
const int kCatTuneTpb[kCatTuneN] = {kFastThreads, 64, 32};
struct CatTune {
    int trials = 0;
    int best_tpb = kFastThreads;
    double rate[kCatTuneN] = {0, 0, 0};
};
std::mutex g_cat_tune_mu;
std::map<std::tuple<int, const void*, int>, CatTune> g_cat_tune;

int cat_blocks_per_sm(int order, int tpb)
{
    int b = 0;
    const cudaError_t e = (order == 1) ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cat_persistent<1>, tpb, 0)
                                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cat_persistent<2>, tpb, 0);
    return (e == cudaSuccess && b > 0) ? b : 1;
}

std::mutex g_plans_mu;
std::map<std::tuple<int, cudaStream_t, int>, CatPlan*> g_plans;
thread_local char g_queue_msg[512] = "";

}  // namespace

const char* catalogue_queue_message() { return g_queue_msg; }

void catalogue_forget_tuned_shape(const void* keys)
{
    std::lock_guard<std::mutex> lock(g_cat_tune_mu);
    for (auto it = g_cat_tune.begin(); it != g_cat_tune.end();) {
        if (std::get<1>(it->first) == keys) it = g_cat_tune.erase(it);
        else ++it;
    }
}

bool catalogue_tuned_shape(int dev, const DevTree& T, int order, int* tpb, double* rates)
{
    std::lock_guard<std::mutex> lock(g_cat_tune_mu);
    auto it = g_cat_tune.find(std::make_tuple(dev, (const void*)T.keys, order));
    if (it == g_cat_tune.end() || it->second.trials < kCatTuneN) return false;
    *tpb = it->second.best_tpb;
    if (rates)
        for (int k = 0; k < kCatTuneN; ++k) rates[k] = it->second.rate[k];
    return true;
}

bool catalogue_persistent_applies(const CatConst& K, bool exact, int order)
{
    return !exact && !K.bundle && !K.born && (order == 1 || order == 2);
}

cudaError_t catalogue_newton_persistent(const DevTree& T, const DevCosmo& Cs, const CatConst& K, const CatRotation* rot,
                                        int order, unsigned nsteps, long long n, const double* d_src, int stride,
                                        double* d_rows, CatRunStats* stats, unsigned* h_status, bool* queue_error,
                                        cudaStream_t stream)
{
    *h_status = 0;
    *queue_error = false;
    std::memset(stats, 0, sizeof(*stats));
    if (n <= 0) return cudaSuccess;
    PropParams P;
    std::memset(&P, 0, sizeof(P));
    P.length = K.length;
    P.max_steps = 100000000ll;
    P.nsteps = nsteps;
    P.order = order;
    P.stop_kind = STOP_R;
    P.nplanes = 1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    CatPlan* plp = nullptr;
    {
        // the plan of this stream: made (graph captured) on its first call and
        // again for a larger batch; calls on one stream are ordered, so only
        // the lookup needs the lock
        std::lock_guard<std::mutex> lock(g_plans_mu);
        CatPlan*& slot = g_plans[std::make_tuple(dev, stream, order)];
        if (slot && slot->cap < n) {
            cudaStreamSynchronize(stream);   // its last launch ran on this stream
            delete slot;
            slot = nullptr;
        }
        if (!slot) {
            CatPlan* fresh = new CatPlan();
            fresh->order = order;
            fresh->cap = std::max<long long>(n, 1 << 16);
            e = plan_build(*fresh, T, Cs, P, K);
            if (e != cudaSuccess) {
                delete fresh;
                return e;
            }
            slot = fresh;
        }
        plp = slot;
    }
    CatPlan& pl = *plp;
    P.ray_stop = pl.D.radius;
    // the call's arguments
    CatCall call;
    call.src = d_src;
    call.rows = d_rows;
    call.n = n;
    call.stride = stride;
    call.has_rot = rot ? 1 : 0;
    if (rot) call.rot = *rot;
    else std::memset(&call.rot, 0, sizeof(call.rot));
    e = cudaMemcpyAsync(pl.d_call, &call, sizeof(call), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    // the persistent kernel's octree, cosmology and parameters for this call
    DevTree Tv = T;
    DevCosmo Cv = Cs;
    CatPlanDev Dv = pl.D;
    CatConst Kv = K;
    void* args[5] = {&Tv, &Cv, &Dv, &P, &Kv};
    cudaKernelNodeParams kp = pl.pparams;
    kp.kernelParams = args;
    kp.extra = nullptr;
    // block size: the tuned one, or this call's candidate while tuning
    static const bool want_tune = !(getenv("MPF_AUTOTUNE") && getenv("MPF_AUTOTUNE")[0] == '0');
    const auto tkey = std::make_tuple(dev, (const void*)T.keys, order);
    int trial = -1, tpb = kFastThreads;
    if (want_tune) {
        std::lock_guard<std::mutex> lock(g_cat_tune_mu);
        CatTune& tu = g_cat_tune[tkey];
        if (tu.trials < kCatTuneN && n >= kCatTuneMin) trial = tu.trials++;
        tpb = (trial >= 0) ? kCatTuneTpb[trial] : tu.best_tpb;
    }
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    kp.blockDim = dim3((unsigned)tpb);
    kp.gridDim = dim3((unsigned)(cat_blocks_per_sm(order, tpb) * sms));
    e = cudaGraphExecKernelNodeSetParams(pl.exec, pl.pnode, &kp);
    if (e != cudaSuccess) return e;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (trial >= 0) {
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
        cudaEventRecord(ev0, stream);
    }
    e = cudaGraphLaunch(pl.exec, stream);
    if (trial >= 0) cudaEventRecord(ev1, stream);
    if (e != cudaSuccess) return e;
    unsigned long long ctl[kQWords], ps[2];
    unsigned cnt[2], st = 0;
    e = cudaMemcpyAsync(ctl, pl.D.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ps, pl.D.psteps, sizeof(ps), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, pl.D.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, pl.D.status, sizeof(st), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (trial >= 0) {
        float ms = 0.f;
        if (e == cudaSuccess && cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess && ms > 0.f) {
            std::lock_guard<std::mutex> lock(g_cat_tune_mu);
            CatTune& tu = g_cat_tune[tkey];
            tu.rate[trial] = (double)ps[0] / (ms * 1e-3);
            if (tu.trials == kCatTuneN) {
                int b = 0;
                for (int k = 1; k < kCatTuneN; ++k)
                    if (tu.rate[k] > tu.rate[b]) b = k;
                tu.best_tpb = kCatTuneTpb[b];
            }
        }
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
    }
    if (e != cudaSuccess) return e;
    stats->rays = (long long)ctl[kQRays];
    stats->photon_steps = (long long)ps[0];
    stats->photon_steps_jacobian = (long long)ps[1];
    stats->iterations = (int)ctl[kQIter];
    stats->launches = pl.kernels;   // the kernels of the one graph launch
    *h_status = st;
    *queue_error = cnt[1] != 0 || ctl[kQHead] != ctl[kQTail];
    if (*queue_error)
        snprintf(g_queue_msg, sizeof(g_queue_msg),
                 "queue head %llu tail %llu in flight %llu, flags %u, %lld sources, capacity %lld; first busy slot at "
                 "position %llu (word %llx, head %llu, tail %llu), first missing item at position %llu (tail %llu)",
                 ctl[kQHead], ctl[kQTail], ctl[kQFlight], cnt[1], n, pl.cap, ctl[kQFault0], ctl[kQFault1], ctl[kQFault2],
                 ctl[kQFault3], ctl[kQFault4], ctl[kQFault5]);
    return cudaSuccess;
}

}  // namespace mpf
