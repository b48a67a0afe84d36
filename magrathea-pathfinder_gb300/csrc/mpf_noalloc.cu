// mpf_propagate_noalloc: the host-buffer propagation call without any device
// allocation.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree while they
// run this path, for example
//  * an application whose device memory is owned by a pooling allocator
//    (PyTorch's caching allocator, a custom arena) that accounts for every
//    byte and must not see foreign allocations fragmenting the pool;
//  * processes sharing one GPU under a hard per-process memory cap (MPS
//    memory limits), where a late allocation can fail;
//  * latency-sensitive loops, where cudaMalloc / cudaFree may synchronise the
//    whole device.
// mpf_propagate allocates device copies of the launch records and the
// outputs, a work-queue counter and a status word on every call; this variant
// stages all of them through one file-scope static device array instead.
//
// Limits and sharing:
//  * the static array is MPF_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that
//    loads the library, held until the process exits;
//  * a call whose staging does not fit is rejected with MPF_BAD_INPUT (split
//    the batch);
//  * every call uses the same array and leaves its last contents there; the
//    queue counter and the status word are cleared at the start of each call;
//    two calls that overlap on the GPU (other host threads, other streams)
//    race on the array, so callers serialise them;
//  * the device address of the array is looked up with cudaGetSymbolAddress
//    the first time the call runs on a device (with that device current);
//    make that first call before any stream capture begins.  The address is
//    kept for the life of the process: it does not survive a cudaDeviceReset
//    of that device (the module, and with it the array, is loaded anew), so
//    a process that resets a device must not call this entry point on it
//    afterwards.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mpf_gb300.h"
#include "mpf_internal.h"

namespace mpf {
cudaError_t launch_propagate_fast_with_queue(const DevTree& T, const DevCosmo& C, const PropParams& P, const double* d_launch,
                                             long long n, const PropOut& O, unsigned long long* queue, cudaStream_t stream);
}

static __device__ __align__(256) unsigned char g_noalloc_scratch[MPF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;
thread_local std::string g_noalloc_err;

int fail(int code, const std::string& msg)
{
    g_noalloc_err = msg;
    return code;
}

// device address of the static array on the current device (set up once)
cudaError_t scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" const char* mpf_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

extern "C" int mpf_propagate_noalloc(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n,
                                     const double* launch, int64_t* steps, double* final_rec, double* plane_rec)
{
    // the same argument rules as mpf_propagate: steps, final_rec and plane_rec may each be NULL
    mpf::PropParams P;
    if (!o || !c || !mpf_internal_fill_params(p, P) || n < 0 || (n > 0 && !launch))
        return fail(MPF_BAD_INPUT, "mpf_propagate_noalloc: bad argument");
    if (n == 0) return MPF_OK;
    const int np = p->nplanes;
    // staging layout: [control 256 B][launch][steps][final][surfaces], 256-B aligned; the
    // kernel writes every ray's step count, so steps are staged even when not copied back
    const size_t b_ctl = 256;
    const size_t b_launch = up256((size_t)n * 6 * sizeof(double));
    const size_t b_steps = up256((size_t)n * sizeof(int64_t));
    const size_t b_final = final_rec ? up256((size_t)n * MPF_PHOTON_FIELDS * sizeof(double)) : 0;
    const size_t b_planes = (plane_rec && np > 0) ? up256((size_t)n * np * MPF_PLANE_FIELDS * sizeof(double)) : 0;
    const size_t need = b_ctl + b_launch + b_steps + b_final + b_planes;
    if (need > (size_t)MPF_NOALLOC_SCRATCH_BYTES)
        return fail(MPF_BAD_INPUT, "mpf_propagate_noalloc: " + std::to_string(n) + " rays need " + std::to_string(need) +
                                       " bytes of staging, more than the " + std::to_string(MPF_NOALLOC_SCRATCH_BYTES) +
                                       "-byte static scratch; split the batch");
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_propagate_noalloc: scratch set-up: ") + cudaGetErrorString(e));
    unsigned char* s = (unsigned char*)base;
    unsigned long long* queue = (unsigned long long*)s;
    unsigned* status = (unsigned*)(s + 64);
    double* d_launch = (double*)(s + b_ctl);
    long long* d_steps = (long long*)(s + b_ctl + b_launch);
    double* d_final = b_final ? (double*)(s + b_ctl + b_launch + b_steps) : nullptr;
    double* d_planes = b_planes ? (double*)(s + b_ctl + b_launch + b_steps + b_final) : nullptr;

    const mpf::DevCosmo C = dev_cosmo(c);
    mpf::PropOut O{d_steps, d_final, d_planes, status, nullptr};

    e = cudaMemset(s, 0, b_ctl);   // queue counter and status word start at zero
    if (e == cudaSuccess) e = cudaMemcpy(d_launch, launch, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice);
    // ORDER = 0 (NGP) runs the float64 kernel in both modes, as in mpf_propagate; that
    // kernel needs no work-queue counter
    if (e == cudaSuccess)
        e = (p->exact || P.order == 0) ? mpf::launch_propagate<true>(o->tree, C, P, d_launch, n, O, 0)
                                       : mpf::launch_propagate_fast_with_queue(o->tree, C, P, d_launch, n, O, queue, 0);
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(st), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && steps) e = cudaMemcpy(steps, d_steps, (size_t)n * sizeof(int64_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && d_final)
        e = cudaMemcpy(final_rec, d_final, (size_t)n * MPF_PHOTON_FIELDS * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && d_planes)
        e = cudaMemcpy(plane_rec, d_planes, (size_t)n * np * MPF_PLANE_FIELDS * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_propagate_noalloc: ") + cudaGetErrorString(e));
    if (st & 1u) return fail(MPF_WARN_MAX_STEPS, "mpf_propagate_noalloc: a ray reached max_steps");
    return MPF_OK;
}
