// Learned field surrogate of the octree gather (per-cone Fourier-feature MLP,
// network in mpf_surrogate.cuh).  It has no counterpart in the reference: it
// stands in for SimpleHyperOctree::tsc / cic (simplehyperoctree.h:1410-1644)
// inside the RK4 stages of Integrator::integrate (integrator.h:648-824), and
// the octree stays its check and fallback.
//
//  * Training samples: points uniform in the cone volume labelled by the
//    octree's TSC gather (the fast-mode record path).
//  * Training: FP32 forward / backward / Adam kernels over batches, the whole
//    step captured once in a CUDA graph and replayed.
//  * Inference: BF16 weights and activations on the tensor cores (tcgen05.mma,
//    accumulators in TMEM, 128 photons per warpgroup tile), FP32 bias + SiLU
//    between layers, fused into the RK4 loop: each thread owns one photon,
//    the four network evaluations of a step (stages 2-4 and the post-step
//    point) are warpgroup-collective.
//  * Every check_every-th step and at the stop, the octree is gathered at the
//    photon's point and the transverse field of both is summed along the path
//    (a checkpointed deflection); a photon whose surrogate deflection drifts
//    from the octree's by more than the tolerance is flagged and, on request,
//    re-run on the plain octree path.
#include <cuda_bf16.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/mpf_gb300.h"
#include "mpf_fast.cuh"
#include "mpf_internal.h"
#include "mpf_surrogate.cuh"
#include "mpf_umma.cuh"

struct mpf_surrogate {
    int device;
    mpf::surr::Spec spec;
    mpf::surr::Cone cone;
    uint64_t seed;
    float* params;          // FP32 master parameters
    float* grads;
    float* adam_m;
    float* adam_v;
    unsigned char* packed;  // inference image
    bool packed_ok;
};

namespace mpf {
namespace surr {

// ---------------------------------------------------------------------------
// shared-memory layout of the tensor-core kernels (one CTA per SM, two
// warpgroups of 128 threads, each with its own activation tile, TMEM columns
// and mbarrier)
// ---------------------------------------------------------------------------
constexpr int kWG = 2;
constexpr int kThreads = 128 * kWG;
constexpr int kActBytes = kWidth * kWidth * 2;
constexpr int kSmemAct = kPackBytes;
constexpr int kSmemBar = kSmemAct + kWG * kActBytes;
constexpr int kSmemSlot = kSmemBar + kWG * 8;
// The allocation covers the reach of an operand descriptor from the last
// tile's last K step with either stride as the row-group stride (start
// 7 x 4 KB, 15 x 2 KB + 128 B beyond), so every operand read stays inside the
// CTA's shared memory.
constexpr int kSmemBytes = kSmemAct + (kWG - 1) * kActBytes + 7 * 4096 + 15 * 2048 + 256;
constexpr uint32_t kTmemCols = 256;            // 128 FP32 columns per warpgroup
constexpr uint64_t kWaitNs = 1000000000ull;    // give up on an MMA after 1 s

static_assert(kPackBytes % 16 == 0, "operand tiles must stay 16-byte aligned");
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");
static_assert(kSmemSlot + 16 <= kSmemBytes, "barriers inside the allocation");

// silu(x) = h + h tanh(h) with h = x / 2, on a pair of values packed as
// bfloat16 (one tanh per pair on the special-function unit, one packed FMA);
// h0, h1 are the halved pre-activations in FP32
__device__ __forceinline__ uint32_t silu2_bf16(float h0, float h1)
{
    const __nv_bfloat162 hh = __floats2bfloat162_rn(h0, h1);
    const uint32_t h = *reinterpret_cast<const uint32_t*>(&hh);
    uint32_t t, y;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(y) : "r"(h), "r"(t));
    return y;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// One warpgroup's view of the network during a tile evaluation.
struct Group {
    unsigned char* sm;      // shared-memory base (packed parameters first)
    unsigned char* act;     // this warpgroup's 128 x 128 activation tile
    uint64_t* bar;
    uint32_t tmem;          // TMEM address of this warpgroup's columns
    uint32_t phase;
    int wg, tid;
    unsigned* err;          // bit 0: an MMA wait ran out
    bool ok;
    bool hold;              // test of the bounded wait: the MMAs are never issued
};

// Copy the packed parameters to shared memory, allocate TMEM, initialise the
// mbarriers.  All threads of the CTA.
__device__ __forceinline__ Group setup(unsigned char* sm, const unsigned char* __restrict__ packed, unsigned* err)
{
    const uint4* src = reinterpret_cast<const uint4*>(packed);
    uint4* dst = reinterpret_cast<uint4*>(sm);
    for (int q = threadIdx.x; q < kPackBytes / 16; q += blockDim.x) dst[q] = __ldg(src + q);
    umma::fence_proxy_async();
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kSmemSlot);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kSmemBar);
    if (threadIdx.x < 32) {
        umma::tmem_alloc(slot, kTmemCols);
        umma::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int w = 0; w < kWG; ++w) umma::mbar_init(bars + w, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    Group g;
    g.sm = sm;
    g.wg = threadIdx.x >> 7;
    g.tid = threadIdx.x & 127;
    g.act = sm + kSmemAct + g.wg * kActBytes;
    g.bar = bars + g.wg;
    g.tmem = *slot + (uint32_t)(g.wg * 128);
    g.phase = 0;
    g.err = err;
    g.ok = true;
    g.hold = false;
    return g;
}

__device__ __forceinline__ void teardown(const Group& g)
{
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (threadIdx.x < 32) umma::tmem_dealloc(*reinterpret_cast<uint32_t*>(g.sm + kSmemSlot), kTmemCols);
}

// Evaluate the network for the warpgroup's 128 rows: thread tid supplies row
// tid's input p (x, y, z, a) and receives its 5 normalised outputs.  Called by
// all 128 threads of the warpgroup with converged warps.
__device__ __forceinline__ void evaluate(Group& g, const Spec& S, const float* p, float* y)
{
    // Fourier features of this row -> BF16 row of the activation tile
    float u[4];
    normalise(S, p, u);
#pragma unroll 1
    for (int j0 = 0; j0 < kFreq; j0 += 8) {
        float sn[8], cs[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) __sincosf(project(S, j0 + q, u), &sn[q], &cs[q]);
        const uint4 vs = make_uint4(pack_bf16(sn[0], sn[1]), pack_bf16(sn[2], sn[3]), pack_bf16(sn[4], sn[5]),
                                    pack_bf16(sn[6], sn[7]));
        const uint4 vc = make_uint4(pack_bf16(cs[0], cs[1]), pack_bf16(cs[2], cs[3]), pack_bf16(cs[4], cs[5]),
                                    pack_bf16(cs[6], cs[7]));
        *reinterpret_cast<uint4*>(g.act + umma::tile_offset(128, g.tid, j0)) = vs;
        *reinterpret_cast<uint4*>(g.act + umma::tile_offset(128, g.tid, kFreq + j0)) = vc;
    }
    const uint32_t lane_base = g.tmem + ((uint32_t)((g.tid >> 5) * 32) << 16);
    const float* bias = reinterpret_cast<const float*>(g.sm + kPackB);
    const float* bias5 = reinterpret_cast<const float*>(g.sm + kPackB5);
#pragma unroll 1
    for (int l = 0; l <= kHidden; ++l) {
        umma::fence_proxy_async();
        umma::bar_sync(1 + g.wg, 128);
        if (g.tid == 0 && g.ok && !g.hold) {
            umma::fence_after_sync();
            const uint32_t a = umma::smem_u32(g.act);
            const int N = (l < kHidden) ? kWidth : kOutPad;
            const uint32_t b = umma::smem_u32(g.sm + ((l < kHidden) ? l * kWidth * kWidth * 2 : kPackW5));
            const uint32_t id = umma::idesc_bf16(128, N);
#pragma unroll
            for (int s = 0; s < kWidth / 16; ++s) umma::mma_bf16(g.tmem, umma::tile_desc(a, 128, s), umma::tile_desc(b, N, s), id, s > 0);
            umma::mma_commit(g.bar);
        }
        bool done = g.ok ? umma::mbar_wait(g.bar, g.phase, kWaitNs) : false;
        g.phase ^= 1u;
        done = __all_sync(0xffffffffu, done);
        if (!done) {
            if (g.ok) atomicOr(g.err, 1u);
            g.ok = false;
        }
        umma::fence_after_sync();
        if (l < kHidden) {
            const float* bl = bias + l * kWidth;
#pragma unroll 1
            for (int c = 0; c < kWidth / 16; ++c) {
                float v[16];
                if (g.ok) umma::tmem_ld16(lane_base + 16 * c, v);
                else
                    for (int q = 0; q < 16; ++q) v[q] = 0.f;
                uint32_t w[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)   // the packed image holds b / 2 for the hidden layers
                    w[q] = silu2_bf16(fmaf(v[2 * q], 0.5f, bl[16 * c + 2 * q]), fmaf(v[2 * q + 1], 0.5f, bl[16 * c + 2 * q + 1]));
                *reinterpret_cast<uint4*>(g.act + umma::tile_offset(128, g.tid, 16 * c)) = make_uint4(w[0], w[1], w[2], w[3]);
                *reinterpret_cast<uint4*>(g.act + umma::tile_offset(128, g.tid, 16 * c + 8)) = make_uint4(w[4], w[5], w[6], w[7]);
            }
        } else {
            float v[16];
            if (g.ok) umma::tmem_ld16(lane_base, v);
            else
                for (int q = 0; q < 16; ++q) v[q] = 0.f;
#pragma unroll
            for (int o = 0; o < kOut; ++o) y[o] = v[o] + bias5[o];
        }
        umma::fence_before_sync();
    }
}

// ---------------------------------------------------------------------------
// inference over a list of points
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1) k_eval(Spec S, const unsigned char* __restrict__ packed,
                                                      const float* __restrict__ in, long long n, float* out, unsigned* err,
                                                      int hold)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    Group g = setup(sm, packed, err);
    g.hold = hold != 0;
    const long long tiles = (n + 127) / 128;
    for (long long t = (long long)blockIdx.x * kWG + g.wg; t < tiles; t += (long long)gridDim.x * kWG) {
        const long long i = t * 128 + g.tid;
        float p[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < n)
            for (int d = 0; d < 4; ++d) p[d] = in[4 * i + d];
        float y[kOut];
        __syncwarp();
        evaluate(g, S, p, y);
        if (i < n)
            for (int o = 0; o < kOut; ++o) out[kOut * i + o] = y[o] * S.stdv[o] + S.mean[o];
    }
    teardown(g);
}

// ---------------------------------------------------------------------------
// fused RK4 propagation with the surrogate in the stages
// ---------------------------------------------------------------------------
struct SurrOut {
    long long* steps;
    double* final_rec;       // n x 28 or null
    unsigned char* flags;    // bit 0: deflection drift above tolerance, bit 1: max steps
    float* drift;            // n, relative checkpointed deflection drift (or null)
    unsigned long long* counters;   // [0] surrogate photon-steps, [1] flagged photons
    unsigned* status;
};

template <int ORDER>
__global__ void __launch_bounds__(kThreads, 1) k_propagate_surrogate(DevTree T, DevCosmo C, PropParams P, Spec S,
                                                                     const unsigned char* __restrict__ packed,
                                                                     const double* __restrict__ launch, long long n,
                                                                     SurrOut O, unsigned long long* queue, unsigned* err,
                                                                     double tol, int check_every)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    Group g = setup(sm, packed, err);
    const double c2 = kC * kC;
    const double mn = -(double)kExtent / 2.0, mx = (double)kExtent / 2.0;
    const double scale = P.length;
    const double inv_scale = 1.0 / scale;
    const double ratio_k = (scale / kC) / P.nsteps;
    const int skind = P.stop_kind;
    const double stop_ref = P.stop_ref;

    bool active = false, exhausted = false;
    long long i = -1, k = 0;
    FastRec b;
    Field7 data;
    Loc here;
    double dl = 0.0, a0 = 1.0, inv_a = 1.0, phi0c2 = 0.0, isw = 0.0, iswold = 0.0, lambda = 0.0, sacc = 0.0;
    int tb = 0;
    float last_data_dt = 0.f, last_dphi = 0.f;
    double last_dl = 1.0;
    double ao[3], as[3], chi_ck = 0.0;   // checkpointed transverse field sums: octree, surrogate
    unsigned flags = 0;

    for (;;) {
        bool finish = false;
        if (!active && !exhausted) {
            const unsigned long long q = atomicAdd(queue, 1ull);
            if (q < (unsigned long long)n) {
                // Integrator::integrate initialisation (integrator.h:678-704), octree field at the start
                i = (long long)q;
                const double* L = launch + 6 * i;
                const double norm0 = sqrt((L[3] - L[0]) * (L[3] - L[0]) + (L[4] - L[1]) * (L[4] - L[1]) + (L[5] - L[2]) * (L[5] - L[2]));
                b.a = 1.0; b.t = 0.0; b.x = L[0]; b.y = L[1]; b.z = L[2]; b.k0 = 1.0;
                b.k1 = (L[3] - L[0]) / norm0; b.k2 = (L[4] - L[1]) / norm0; b.k3 = (L[5] - L[2]) / norm0;
                here = locate_full(T, b.x, b.y, b.z);
                data = gather_at<ORDER>(T, here, PosAt{b.x, b.y, b.z}, true, nullptr, 0, true);
                const double ph = (double)data.phi / c2;
                const double nk = sqrt((c2 * (1.0 + 2.0 * ph) * b.k0 * b.k0) / ((1.0 - 2.0 * ph) * (b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3)));
                b.k1 *= nk; b.k2 *= nk; b.k3 *= nk;
                b.a = interp_fast(C, b.t, C.a, C.slope_a);
                b.level = (here.cell >= 0) ? here.level : 0;
                b.ah = 0.f;   // integrator.h:684-685 overwrites data.a() with zero at the start
                b.rho = data.rho; b.phi = data.phi; b.dx = data.dx; b.dy = data.dy; b.dz = data.dz; b.dt = data.dt;
                b.red = 0.0; b.isw = 0.0; b.chi = 0.0; b.iswold = 0.0; b.lambda = 0.0; b.s = 0.0;
                dl = (here.cell >= 0 ? cell_extent(here.level) : 0.0) * (b.a * b.a * ratio_k);
                a0 = b.a;
                inv_a = recip(b.a);
                tb = bracket_lut(C, b.t);
                phi0c2 = b.phi / c2;
                last_data_dt = data.dt; last_dphi = 0.f; last_dl = 1.0;
                isw = iswold = lambda = sacc = 0.0;
                k = 0;
                flags = 0;
                for (int d = 0; d < 3; ++d) ao[d] = as[d] = 0.0;
                chi_ck = 0.0;
                active = true;
                if (is_empty(data)) finish = true;
            } else {
                exhausted = true;
            }
        }
        __syncwarp();
        if (!umma::bar_or(1 + g.wg, 128, active)) break;

        // ---- one RK4 step: stage 1 from the field at b, stages 2-4 and the
        // post-step point from the network
        double bc[9], core[9], dc[9], acc[9];
        float kfs[3];
        double p9[9];
        const bool run = active && !finish;
        if (run) {
            bc[0] = b.a; bc[1] = b.t; bc[2] = b.x; bc[3] = b.y; bc[4] = b.z;
            bc[5] = b.k0; bc[6] = b.k1; bc[7] = b.k2; bc[8] = b.k3;
            if (k >= P.max_steps) {
                flags |= 2u;
                finish = true;
            } else {
                rhs_math(C, data, bc, inv_a, tb, dc, kfs);
                const double cs = 0.5 * dl;
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    acc[q] = dc[q];
                    core[q] = bc[q] + ((q >= 2 && q <= 4) ? cs * inv_scale : cs) * dc[q];
                }
            }
        }
#pragma unroll 1
        for (int sg = 1; sg <= 4; ++sg) {
            const bool live = active && !finish;
            float pin[4] = {0.f, 0.f, 0.f, 0.f};
            if (live) {
                const double* src = (sg < 4) ? core : p9;
                pin[0] = (float)src[2]; pin[1] = (float)src[3]; pin[2] = (float)src[4]; pin[3] = (float)src[0];
            }
            float y[kOut];
            __syncwarp();
            evaluate(g, S, pin, y);
            if (!live) continue;
            Field7 f;
            f.phi = fmaf(y[0], S.stdv[0], S.mean[0]);
            f.dx = fmaf(y[1], S.stdv[1], S.mean[1]);
            f.dy = fmaf(y[2], S.stdv[2], S.mean[2]);
            f.dz = fmaf(y[3], S.stdv[3], S.mean[3]);
            f.dt = fmaf(y[4], S.stdv[4], S.mean[4]);
            f.rho = 0.f;
            f.a = 0.f;
            if (sg < 4) {
                rhs_math(C, f, core, recip(core[0]), tb, dc, kfs);
                if (sg < 3) {
                    const double cs = (sg == 1) ? 0.5 * dl : dl;
#pragma unroll
                    for (int q = 0; q < 9; ++q) {
                        acc[q] += 2.0 * dc[q];
                        core[q] = bc[q] + ((q >= 2 && q <= 4) ? cs * inv_scale : cs) * dc[q];
                    }
                } else {
                    const double dl6 = dl * (1.0 / 6.0), dl6p = dl6 * inv_scale;
#pragma unroll
                    for (int q = 0; q < 9; ++q) p9[q] = bc[q] + ((q >= 2 && q <= 4) ? dl6p : dl6) * (acc[q] + dc[q]);
                }
            } else {
                // post-step point (integrator.h:740-776)
                FastRec p;
                p.a = p9[0]; p.t = p9[1]; p.x = p9[2]; p.y = p9[3]; p.z = p9[4];
                p.k0 = p9[5]; p.k1 = p9[6]; p.k2 = p9[7]; p.k3 = p9[8];
                const Loc ploc = locate_near(T, here, p.x, p.y, p.z);
                const uint32_t last = (ploc.cell >= 0) ? (uint32_t)((1ull << ploc.level) - 1ull) : 0u;
                const bool face = (ploc.cell < 0) || ploc.c[0] == 0u || ploc.c[1] == 0u || ploc.c[2] == 0u ||
                                  ploc.c[0] >= last || ploc.c[1] >= last || ploc.c[2] >= last;
                const bool outside = (ploc.cell < 0) || p.a < 0.0 ||
                                     (face && !((p.x > mn) && (p.x < mx) && (p.y > mn) && (p.y < mx) && (p.z > mn) && (p.z < mx)));
                if (outside) {
                    finish = true;
                } else {
                    data = f;
                    p.level = ploc.level;
                    p.ah = 0.f;
                    p.rho = 0.f; p.phi = f.phi; p.dx = f.dx; p.dy = f.dy; p.dz = f.dz;
                    p.dt = -f.dt;
                    const float dphi_last = f.phi - (float)b.phi;
                    const double dl_last = dl;
                    isw += (double)(b.dt + p.dt) * (p.t - b.t) * (1.0 / c2);
                    if (O.final_rec) {
                        iswold -= 2.0 * (p.phi - b.phi) * (1.0 / c2) -
                                  (((double)b.dx + (double)p.dx) * (p.x - b.x) * scale + ((double)b.dy + (double)p.dy) * (p.y - b.y) * scale +
                                   ((double)b.dz + (double)p.dz) * (p.z - b.z) * scale) * (1.0 / c2);
                    }
                    p.chi = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
                    lambda += dl;
                    sacc += (double)sqrtf((float)((p.x - b.x) * (p.x - b.x) + (p.y - b.y) * (p.y - b.y) + (p.z - b.z) * (p.z - b.z)));
                    const double inv_pa = recip(p.a);
                    p.red = a0 * inv_pa * (1.0 + phi0c2 - p.phi * (1.0 / c2)) - 1.0;
                    p.isw = isw; p.iswold = iswold; p.lambda = lambda; p.s = sacc;
                    dl = cell_extent(ploc.level) * (p.a * p.a * ratio_k);
                    last_data_dt = f.dt;
                    last_dphi = dphi_last;
                    last_dl = dl_last;
                    here = ploc;
                    ++k;
                    if (check_every > 0 && (k % check_every) == 0) {
                        // checkpoint: the octree's field at the same point
                        const Field7 go = gather_at<ORDER>(T, here, PosAt{p.x, p.y, p.z}, false, nullptr, 0, false);
                        const double kn = rsqrt(p.k1 * p.k1 + p.k2 * p.k2 + p.k3 * p.k3);
                        const double nx = p.k1 * kn, ny = p.k2 * kn, nz = p.k3 * kn;
                        const double w = p.chi - chi_ck;
                        const double so = go.dx * nx + go.dy * ny + go.dz * nz, ss = f.dx * nx + f.dy * ny + f.dz * nz;
                        ao[0] += (go.dx - so * nx) * w; ao[1] += (go.dy - so * ny) * w; ao[2] += (go.dz - so * nz) * w;
                        as[0] += (f.dx - ss * nx) * w; as[1] += (f.dy - ss * ny) * w; as[2] += (f.dz - ss * nz) * w;
                        chi_ck = p.chi;
                    }
                    b = p;
                    inv_a = inv_pa;
                    bool stop;
                    switch (skind) {
                    case STOP_R: stop = b.chi > stop_ref; break;
                    case STOP_LAMBDA: stop = b.lambda > stop_ref; break;
                    case STOP_REDSHIFT: stop = b.red > stop_ref; break;
                    case STOP_T: stop = b.t > stop_ref; break;
                    case STOP_A: stop = b.a < stop_ref; break;
                    case STOP_PLANE: stop = (b.x * P.ki[0] + b.y * P.ki[1] + b.z * P.ki[2]) > stop_ref; break;
                    case STOP_S: stop = b.s > stop_ref; break;
                    default: stop = true;
                    }
                    if (stop) finish = true;
                }
            }
        }
        if (active && finish) {
            // final checkpoint at the last accepted point, then the drift test
            if (k > 0 && here.cell >= 0 && b.chi > chi_ck) {
                const Field7 go = gather_at<ORDER>(T, here, PosAt{b.x, b.y, b.z}, false, nullptr, 0, false);
                const double kn = rsqrt(b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3);
                const double nx = b.k1 * kn, ny = b.k2 * kn, nz = b.k3 * kn;
                const double w = b.chi - chi_ck;
                const double so = go.dx * nx + go.dy * ny + go.dz * nz, ss = b.dx * nx + b.dy * ny + b.dz * nz;
                ao[0] += (go.dx - so * nx) * w; ao[1] += (go.dy - so * ny) * w; ao[2] += (go.dz - so * nz) * w;
                as[0] += (b.dx - ss * nx) * w; as[1] += (b.dy - ss * ny) * w; as[2] += (b.dz - ss * nz) * w;
            }
            const double dn = sqrt((as[0] - ao[0]) * (as[0] - ao[0]) + (as[1] - ao[1]) * (as[1] - ao[1]) + (as[2] - ao[2]) * (as[2] - ao[2]));
            const double an = sqrt(ao[0] * ao[0] + ao[1] * ao[1] + ao[2] * ao[2]);
            const double drift = (an > 0.0) ? dn / an : (dn > 0.0 ? 1e30 : 0.0);
            if (!(drift <= tol)) flags |= 1u;
            long long size = k + 1;
            if (signbit(b.red) || signbit(b.a)) size -= 1;
            O.steps[i] = size;
            if (O.drift) O.drift[i] = (float)drift;
            O.flags[i] = (unsigned char)flags;
            if (O.final_rec) {
                double* o = O.final_rec + i * kPhotonFields;
                if (size == k + 1) {
                    Rec r;
                    r.a = b.a; r.t = b.t; r.x = b.x; r.y = b.y; r.z = b.z; r.k0 = b.k0; r.k1 = b.k1; r.k2 = b.k2; r.k3 = b.k3;
                    r.level = b.level; r.ah = b.ah; r.rho = b.rho; r.phi = b.phi;
                    r.dx = b.dx; r.dy = b.dy; r.dz = b.dz; r.dt = b.dt;
                    r.dphidl = (k > 0) ? ((double)last_data_dt * b.k0 + ((double)b.dx * b.k1 + (double)b.dy * b.k2 + (double)b.dz * b.k3)) : 0.0;
                    r.lap = (k > 0) ? (double)last_dphi / last_dl : 0.0;
                    const double kk = b.k1 * b.k1 + b.k2 * b.k2 + b.k3 * b.k3;
                    r.ds2 = (b.a * b.a) * (-(c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0) + ((1.0 - 2.0 * (b.phi / c2)) * kk));
                    r.err = 1.0 - ((1.0 - 2.0 * (b.phi / c2)) * kk) / (c2 * (1.0 + 2.0 * (b.phi / c2)) * b.k0 * b.k0);
                    r.red = b.red; r.isw = b.isw; r.iswold = b.iswold; r.chi = b.chi; r.lambda = b.lambda; r.s = b.s;
                    r.index = (double)k;
                    write_rec(o, r);
                } else {
                    for (int q = 0; q < kPhotonFields; ++q) o[q] = 0.0;
                }
            }
            atomicAdd(O.counters, (unsigned long long)k);
            if (flags & 1u) atomicAdd(O.counters + 1, 1ull);
            if (flags & 2u) atomicOr(O.status, 1u);
            active = false;
        }
    }
    teardown(g);
}

// ---------------------------------------------------------------------------
// training
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t splitmix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ double unit(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

// Samples uniform in the cone volume, labelled by the octree's TSC gather.
// Sample index = *step * n + first + b.  x: n x 4 (x y z a), t: n x 5 raw
// (phi dphidx dphidy dphidz dphidt) or normalised by S when norm != 0.
__global__ void k_sample(DevTree T, Cone K, Spec S, uint64_t seed, const long long* __restrict__ step, long long first,
                         long long n, int norm, float* x, float* t)
{
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint64_t idx = (uint64_t)((step ? *step : 0ll) * n + first + b);
    const uint64_t h0 = splitmix(seed ^ (idx * 0xD1B54A32D192ED03ull));
    const uint64_t h1 = splitmix(h0), h2 = splitmix(h1);
    const double r0 = K.r_min * K.r_min * K.r_min, r1 = K.r_max * K.r_max * K.r_max;
    const double px = cbrt(r0 + unit(h0) * (r1 - r0));
    const double py = px * K.tan_y * (2.0 * unit(h1) - 1.0);
    const double pz = px * K.tan_z * (2.0 * unit(h2) - 1.0);
    const Loc d = locate_full(T, px, py, pz);
    const Field7 f = gather_at<2>(T, d, PosAt{px, py, pz}, true, nullptr, 0, false);
    x[4 * b] = (float)px; x[4 * b + 1] = (float)py; x[4 * b + 2] = (float)pz; x[4 * b + 3] = f.a;
    const float v[kOut] = {f.phi, f.dx, f.dy, f.dz, f.dt};
    for (int o = 0; o < kOut; ++o) t[kOut * b + o] = norm ? (v[o] - S.mean[o]) / S.stdv[o] : v[o];
}

// FP32 Fourier features h0 (n x 128) of raw inputs (n x 4)
__global__ void k_features(Spec S, const float* __restrict__ x, long long n, float* h0)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * kFreq) return;
    const long long b = idx / kFreq;
    const int j = (int)(idx % kFreq);
    float p[4] = {x[4 * b], x[4 * b + 1], x[4 * b + 2], x[4 * b + 3]};
    float u[4];
    normalise(S, p, u);
    float sn, cs;
    __sincosf(project(S, j, u), &sn, &cs);
    h0[b * kWidth + j] = sn;
    h0[b * kWidth + kFreq + j] = cs;
}

__device__ __forceinline__ float silu_exact(float z) { return z / (1.f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.f / (1.f + expf(-z));
    return s * (1.f + z * (1.f - s));
}

// C[m][n] (op)= sum_k A(m, k) B(n, k), A(m, k) = A[m sam + k sak], B(n, k) = B[n sbn + k sbk].
// EPI 0: C = acc + bias, H = silu(C);  1: C = acc + bias;  2: C = acc * silu'(Z);
// 3: C += acc (atomic; blockIdx.z splits K in chunks of kchunk).
constexpr int kTM = 64, kTN = 64, kTK = 16;
template <int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, long long sam, long long sak,
                                              const float* __restrict__ B, long long sbn, long long sbk, float* C, int ldc,
                                              const float* __restrict__ bias, float* H, const float* __restrict__ Z, int kchunk)
{
    __shared__ float As[kTK][kTM + 4];
    __shared__ float Bs[kTK][kTN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = kb; k0 < ke; k0 += kTK) {
        for (int e = threadIdx.x; e < kTM * kTK; e += 256) {
            int mm, kk;
            if (sak == 1) { kk = e % kTK; mm = e / kTK; } else { mm = e % kTM; kk = e / kTM; }
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < ke) ? A[m * sam + k * sak] : 0.f;
        }
        for (int e = threadIdx.x; e < kTN * kTK; e += 256) {
            int nn, kk;
            if (sbk == 1) { kk = e % kTK; nn = e / kTK; } else { nn = e % kTN; kk = e / kTN; }
            const int nidx = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (nidx < N && k < ke) ? B[nidx * sbn + k * sbk] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTK; ++kk) {
            float a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int nn = n0 + tx * 4 + j;
            if (nn >= N) continue;
            const long long o = (long long)m * ldc + nn;
            if (EPI == 0) {
                const float z = acc[i][j] + bias[nn];
                C[o] = z;
                H[o] = silu_exact(z);
            } else if (EPI == 1) {
                C[o] = acc[i][j] + bias[nn];
            } else if (EPI == 2) {
                C[o] = acc[i][j] * dsilu(Z[o]);
            } else {
                atomicAdd(C + o, acc[i][j]);
            }
        }
    }
}

// loss = mean over rows and the 5 outputs of (y - t)^2; dy = its gradient
__global__ void k_loss(long long n, const float* __restrict__ y, const float* __restrict__ t, float* dy, double* loss,
                       const long long* __restrict__ step)
{
    __shared__ double part[256];
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (b < n) {
        const float sc = 2.f / (float)(n * kOut);
        for (int o = 0; o < kOut; ++o) {
            const float d = y[b * kOutPad + o] - t[b * kOut + o];
            l += (double)d * d;
            dy[b * kOutPad + o] = sc * d;
        }
    }
    part[threadIdx.x] = l;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss + (step ? *step : 0ll), part[0] / (double)(n * kOut));
}

// column sums of D (n x N, leading dimension ld) added into out[N]
__global__ void k_colsum(long long n, int N, const float* __restrict__ D, int ld, float* out)
{
    __shared__ float part[256];
    const int col = blockIdx.x;
    float s = 0.f;
    for (long long r = (long long)blockIdx.y * 256 + threadIdx.x; r < n; r += (long long)gridDim.y * 256) s += D[r * ld + col];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int q = 128; q > 0; q >>= 1) {
        if (threadIdx.x < q) part[threadIdx.x] += part[threadIdx.x + q];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out + col, part[0]);
}

// Adam with bias correction and a cosine learning-rate decay to lr / 100
__global__ void k_adam(int np, float* w, const float* __restrict__ g, float* m, float* v, const long long* __restrict__ step,
                       double lr0, long long total)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long t = *step + 1;
    const double frac = fmin(1.0, (double)t / (double)(total > 0 ? total : 1));
    const float lr = (float)(lr0 * (0.01 + 0.99 * 0.5 * (1.0 + cos(3.141592653589793 * frac))));
    const float b1 = 0.9f, b2 = 0.999f;
    const float gi = g[q];
    const float mi = b1 * m[q] + (1.f - b1) * gi;
    const float vi = b2 * v[q] + (1.f - b2) * gi * gi;
    m[q] = mi;
    v[q] = vi;
    const float mh = mi / (1.f - powf(b1, (float)t)), vh = vi / (1.f - powf(b2, (float)t));
    w[q] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

__global__ void k_step_inc(long long* step) { *step += 1; }

// FP32 parameters -> inference image (BF16 tiles in the operand layout; FP32
// biases, those of the hidden layers halved for silu2_bf16)
__global__ void k_pack(const float* __restrict__ prm, unsigned char* out)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < kHidden * kWidth * kWidth) {
        const int l = q / (kWidth * kWidth), r = (q / kWidth) % kWidth, c = q % kWidth;
        const float w = prm[l * kLayerStride + r * kWidth + c];
        *reinterpret_cast<__nv_bfloat16*>(out + l * kWidth * kWidth * 2 + umma::tile_offset(kWidth, r, c)) = __float2bfloat16_rn(w);
    }
    if (q < kOutPad * kWidth) {
        const int r = q / kWidth, c = q % kWidth;
        *reinterpret_cast<__nv_bfloat16*>(out + kPackW5 + umma::tile_offset(kOutPad, r, c)) = __float2bfloat16_rn(prm[kW5 + q]);
    }
    if (q < kHidden * kWidth) {
        const int l = q / kWidth, c = q % kWidth;
        reinterpret_cast<float*>(out + kPackB)[q] = 0.5f * prm[l * kLayerStride + kWidth * kWidth + c];   // halved: see silu2_bf16
    }
    if (q < kOutPad) reinterpret_cast<float*>(out + kPackB5)[q] = prm[kB5 + q];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Buffers {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    float* f(size_t count)
    {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, count * sizeof(float));
        if (p) ptrs.push_back(p);
        return (float*)p;
    }
    template <class Tp>
    Tp* any(size_t bytes)
    {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, bytes);
        if (p) ptrs.push_back(p);
        return (Tp*)p;
    }
    ~Buffers()
    {
        for (void* p : ptrs) cudaFree(p);
    }
};

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// Forward and backward over one batch of n rows: features, 4 hidden layers,
// output, loss and all parameter gradients (added into grads).
struct Batch {
    long long n;
    float *x, *t, *h[kHidden + 1], *z[kHidden], *y, *dy, *d0, *d1;
};

static int enqueue_forward_backward(const Spec& S, const float* prm, float* grads, Batch& B, double* loss,
                                    const long long* step, cudaStream_t s)
{
    int launches = 0;
    const long long n = B.n;
    k_features<<<blocks_for(n * kFreq, 256), 256, 0, s>>>(S, B.x, n, B.h[0]);
    ++launches;
    const dim3 grid_h(kWidth / kTN, blocks_for(n, kTM), 1);
    for (int l = 0; l < kHidden; ++l) {
        k_gemm<0><<<grid_h, 256, 0, s>>>((int)n, kWidth, kWidth, B.h[l], kWidth, 1, prm + l * kLayerStride, kWidth, 1, B.z[l],
                                         kWidth, prm + l * kLayerStride + kWidth * kWidth, B.h[l + 1], nullptr, kWidth);
        ++launches;
    }
    k_gemm<1><<<dim3(1, blocks_for(n, kTM), 1), 256, 0, s>>>((int)n, kOutPad, kWidth, B.h[kHidden], kWidth, 1, prm + kW5, kWidth, 1,
                                                            B.y, kOutPad, prm + kB5, nullptr, nullptr, kWidth);
    k_loss<<<blocks_for(n, 256), 256, 0, s>>>(n, B.y, B.t, B.dy, loss, step);
    launches += 2;
    // output layer: dW5 = dy^T h4, db5 = colsum(dy), d(h4) = dy W5 -> dz4
    const int kchunk = 256;
    const unsigned ksplit = blocks_for(n, kchunk);
    k_gemm<3><<<dim3(kWidth / kTN, 1, ksplit), 256, 0, s>>>(kOutPad, kWidth, (int)n, B.dy, 1, kOutPad, B.h[kHidden], 1, kWidth,
                                                            grads + kW5, kWidth, nullptr, nullptr, nullptr, kchunk);
    k_colsum<<<dim3(kOutPad, std::min(64u, blocks_for(n, 256))), 256, 0, s>>>(n, kOutPad, B.dy, kOutPad, grads + kB5);
    k_gemm<2><<<grid_h, 256, 0, s>>>((int)n, kWidth, kOutPad, B.dy, kOutPad, 1, prm + kW5, 1, kWidth, B.d0, kWidth, nullptr,
                                     nullptr, B.z[kHidden - 1], kWidth);
    launches += 3;
    float* dz = B.d0;
    float* other = B.d1;
    for (int l = kHidden - 1; l >= 0; --l) {
        float* gW = grads + l * kLayerStride;
        k_gemm<3><<<dim3(kWidth / kTN, kWidth / kTM, ksplit), 256, 0, s>>>(kWidth, kWidth, (int)n, dz, 1, kWidth, B.h[l], 1, kWidth,
                                                                           gW, kWidth, nullptr, nullptr, nullptr, kchunk);
        k_colsum<<<dim3(kWidth, std::min(64u, blocks_for(n, 256))), 256, 0, s>>>(n, kWidth, dz, kWidth, gW + kWidth * kWidth);
        launches += 2;
        if (l > 0) {
            k_gemm<2><<<grid_h, 256, 0, s>>>((int)n, kWidth, kWidth, dz, kWidth, 1, prm + l * kLayerStride, 1, kWidth, other, kWidth,
                                             nullptr, nullptr, B.z[l - 1], kWidth);
            ++launches;
            std::swap(dz, other);
        }
    }
    return launches;
}

static bool alloc_batch(Buffers& mem, Batch& B, long long n)
{
    B.n = n;
    B.x = mem.f((size_t)n * 4);
    B.t = mem.f((size_t)n * kOut);
    for (int l = 0; l <= kHidden; ++l) B.h[l] = mem.f((size_t)n * kWidth);
    for (int l = 0; l < kHidden; ++l) B.z[l] = mem.f((size_t)n * kWidth);
    B.y = mem.f((size_t)n * kOutPad);
    B.dy = mem.f((size_t)n * kOutPad);
    B.d0 = mem.f((size_t)n * kWidth);
    B.d1 = mem.f((size_t)n * kWidth);
    if (mem.err == cudaSuccess) mem.err = cudaMemset(B.dy, 0, (size_t)n * kOutPad * sizeof(float));
    return mem.err == cudaSuccess;
}

static cudaError_t set_smem_attrs()
{
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_propagate_surrogate<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_propagate_surrogate<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e == cudaSuccess) done = true;
    return e;
}

static int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

}  // namespace surr
}  // namespace mpf

// ===========================================================================
// C ABI
// ===========================================================================
using namespace mpf::surr;

namespace {

int fail(int code, const std::string& m) { return mpf_internal_set_error(code, m.c_str()); }
int cuda_fail(cudaError_t e, const char* where)
{
    return fail(e == cudaErrorMemoryAllocation ? MPF_OUT_OF_MEMORY : MPF_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}

int pack(mpf_surrogate* s)
{
    k_pack<<<blocks_for(kHidden * kWidth * kWidth, 256), 256>>>(s->params, s->packed);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate: pack");
    s->packed_ok = true;
    return MPF_OK;
}

}  // namespace

extern "C" {

int mpf_surrogate_create(const mpf_surrogate_domain* d, mpf_surrogate** out)
{
    if (!d || !out || !(d->r_max > d->r_min) || !(d->r_min >= 0.0) || !(d->tan_half[0] > 0.0) || !(d->tan_half[1] > 0.0) ||
        !(d->a_max > d->a_min))
        return fail(MPF_BAD_INPUT, "mpf_surrogate_create: bad domain");
    for (int q = 0; q < 4; ++q)
        if (!(d->freq_sigma[q] >= 0.0)) return fail(MPF_BAD_INPUT, "mpf_surrogate_create: bad frequency scale");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(MPF_NO_DEVICE, "mpf_surrogate_create: no CUDA device");
    mpf_surrogate* s = new mpf_surrogate();
    cudaGetDevice(&s->device);
    s->seed = d->seed;
    s->cone = Cone{d->tan_half[0], d->tan_half[1], d->r_min, d->r_max};
    Spec& S = s->spec;
    const double lo[4] = {0.0, -d->r_max * d->tan_half[0], -d->r_max * d->tan_half[1], d->a_min};
    const double hi[4] = {d->r_max, d->r_max * d->tan_half[0], d->r_max * d->tan_half[1], d->a_max};
    for (int q = 0; q < 4; ++q) {
        S.lo[q] = (float)lo[q];
        S.sc[q] = (float)(2.0 / (hi[q] - lo[q]));
    }
    std::mt19937_64 rng(d->seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int j = 0; j < kFreq; ++j)
        for (int q = 0; q < 4; ++q) S.freq[j][q] = (float)(M_PI * d->freq_sigma[q] * nd(rng));
    for (int o = 0; o < kOut; ++o) {
        S.mean[o] = 0.f;
        S.stdv[o] = 1.f;
    }
    // LeCun-normal weights, zero biases; output rows 5..15 stay zero
    std::vector<float> prm(kParams, 0.f);
    for (int l = 0; l < kHidden; ++l)
        for (int q = 0; q < kWidth * kWidth; ++q) prm[l * kLayerStride + q] = (float)(nd(rng) / std::sqrt((double)kWidth));
    for (int q = 0; q < kOut * kWidth; ++q) prm[kW5 + q] = (float)(nd(rng) / std::sqrt((double)kWidth));
    cudaError_t e = cudaMalloc(&s->params, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->grads, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->adam_m, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->adam_v, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->packed, kPackBytes);
    if (e == cudaSuccess) e = cudaMemcpy(s->params, prm.data(), kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->adam_m, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(s->adam_v, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(s->packed, 0, kPackBytes);
    if (e != cudaSuccess) {
        mpf_surrogate_destroy(s);
        return cuda_fail(e, "mpf_surrogate_create");
    }
    const int rc = pack(s);
    if (rc != MPF_OK) {
        mpf_surrogate_destroy(s);
        return rc;
    }
    *out = s;
    return MPF_OK;
}

void mpf_surrogate_destroy(mpf_surrogate* s)
{
    if (!s) return;
    cudaFree(s->params);
    cudaFree(s->grads);
    cudaFree(s->adam_m);
    cudaFree(s->adam_v);
    cudaFree(s->packed);
    delete s;
}

int mpf_surrogate_get_params(const mpf_surrogate* s, float* params, float* norm)
{
    if (!s) return fail(MPF_BAD_INPUT, "mpf_surrogate_get_params: null handle");
    if (params) {
        const cudaError_t e = cudaMemcpy(params, s->params, kParams * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_get_params");
    }
    if (norm) std::memcpy(norm, &s->spec, sizeof(Spec));
    return MPF_OK;
}

int mpf_surrogate_set_params(mpf_surrogate* s, const float* params, const float* norm)
{
    if (!s) return fail(MPF_BAD_INPUT, "mpf_surrogate_set_params: null handle");
    if (norm) {
        Spec S;
        std::memcpy(&S, norm, sizeof(Spec));
        for (int o = 0; o < kOut; ++o)
            if (!(S.stdv[o] > 0.f)) return fail(MPF_BAD_INPUT, "mpf_surrogate_set_params: output scales must be positive");
        s->spec = S;
    }
    if (params) {
        const cudaError_t e = cudaMemcpy(s->params, params, kParams * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_set_params");
        return pack(s);
    }
    return MPF_OK;
}

int mpf_surrogate_sample(const mpf_surrogate* s, const mpf_octree* o, uint64_t first, int64_t n, float* inputs, float* targets)
{
    if (!s || !o || n < 0 || (n > 0 && (!inputs || !targets))) return fail(MPF_BAD_INPUT, "mpf_surrogate_sample: bad argument");
    if (n == 0) return MPF_OK;
    Buffers mem;
    float* x = mem.f((size_t)n * 4);
    float* t = mem.f((size_t)n * kOut);
    if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_sample");
    k_sample<<<blocks_for(n, 128), 128>>>(o->tree, s->cone, s->spec, s->seed, nullptr, (long long)first, n, 0, x, t);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(inputs, x, (size_t)n * 4 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(targets, t, (size_t)n * kOut * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_sample");
    return MPF_OK;
}

int mpf_surrogate_loss_grad(mpf_surrogate* s, int64_t n, const float* inputs, const float* targets, double* loss, float* grad)
{
    if (!s || n <= 0 || !inputs || !targets) return fail(MPF_BAD_INPUT, "mpf_surrogate_loss_grad: bad argument");
    Buffers mem;
    Batch B;
    if (!alloc_batch(mem, B, n)) return cuda_fail(mem.err, "mpf_surrogate_loss_grad");
    double* dloss = mem.any<double>(sizeof(double));
    if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_loss_grad");
    // normalised targets
    std::vector<float> tn((size_t)n * kOut);
    for (int64_t b = 0; b < n; ++b)
        for (int q = 0; q < kOut; ++q) tn[b * kOut + q] = (targets[b * kOut + q] - s->spec.mean[q]) / s->spec.stdv[q];
    cudaError_t e = cudaMemcpy(B.x, inputs, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(B.t, tn.data(), tn.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->grads, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(dloss, 0, sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_loss_grad");
    enqueue_forward_backward(s->spec, s->params, s->grads, B, dloss, nullptr, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess && grad) e = cudaMemcpy(grad, s->grads, kParams * sizeof(float), cudaMemcpyDeviceToHost);
    double hl = 0.0;
    if (e == cudaSuccess) e = cudaMemcpy(&hl, dloss, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_loss_grad");
    if (loss) *loss = hl;
    return MPF_OK;
}

int mpf_surrogate_train(mpf_surrogate* s, const mpf_octree* o, const mpf_surrogate_train_params* p, mpf_surrogate_train_stats* st)
{
    if (!s || !o || !p || p->batch < 256 || p->samples < p->batch || !(p->lr > 0.0) || p->stat_samples < 2)
        return fail(MPF_BAD_INPUT, "mpf_surrogate_train: bad argument");
    const long long nb = p->batch;
    const long long steps = p->samples / nb;
    Buffers mem;
    // output normalisation from a first, separate set of samples
    {
        const long long ns = p->stat_samples;
        float* x = mem.f((size_t)ns * 4);
        float* t = mem.f((size_t)ns * kOut);
        if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_train");
        const uint64_t stats_first = 0x5A5A5A5A5A5A5A5Aull;   // disjoint from the training stream's indices
        k_sample<<<blocks_for(ns, 128), 128>>>(o->tree, s->cone, s->spec, s->seed, nullptr, (long long)stats_first, ns, 0, x, t);
        std::vector<float> h((size_t)ns * kOut);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), t, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_train: statistics");
        for (int q = 0; q < kOut; ++q) {
            double m = 0.0, v = 0.0;
            for (long long b = 0; b < ns; ++b) m += h[b * kOut + q];
            m /= (double)ns;
            for (long long b = 0; b < ns; ++b) v += (h[b * kOut + q] - m) * (h[b * kOut + q] - m);
            v /= (double)(ns - 1);
            s->spec.mean[q] = (float)m;
            s->spec.stdv[q] = (float)(v > 0.0 ? std::sqrt(v) : 1.0);
        }
    }
    Batch B;
    if (!alloc_batch(mem, B, nb)) return cuda_fail(mem.err, "mpf_surrogate_train");
    long long* dstep = mem.any<long long>(sizeof(long long));
    double* dloss = mem.any<double>((size_t)steps * sizeof(double));
    if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_train");
    cudaError_t e = cudaMemset(dstep, 0, sizeof(long long));
    if (e == cudaSuccess) e = cudaMemset(dloss, 0, (size_t)steps * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(s->adam_m, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(s->adam_v, 0, kParams * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_train");
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_train: stream");
    // one training step, captured once
    int launches = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(s->grads, 0, kParams * sizeof(float), cs);
        k_sample<<<blocks_for(nb, 128), 128, 0, cs>>>(o->tree, s->cone, s->spec, s->seed, dstep, 0, nb, 1, B.x, B.t);
        launches = 1 + enqueue_forward_backward(s->spec, s->params, s->grads, B, dloss, dstep, cs);
        k_adam<<<blocks_for(kParams, 256), 256, 0, cs>>>(kParams, s->params, s->grads, s->adam_m, s->adam_v, dstep, p->lr, steps);
        k_step_inc<<<1, 1, 0, cs>>>(dstep);
        launches += 2;
        e = cudaStreamEndCapture(cs, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    const auto t0 = std::chrono::steady_clock::now();
    for (long long q = 0; q < steps && e == cudaSuccess; ++q) e = cudaGraphLaunch(exec, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    const auto t1 = std::chrono::steady_clock::now();
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_train");
    std::vector<double> hl((size_t)steps);
    e = cudaMemcpy(hl.data(), dloss, (size_t)steps * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_train");
    const int rc = pack(s);
    if (rc != MPF_OK) return rc;
    if (st) {
        const long long w = std::max(1ll, steps / 100);
        double f = 0.0, l = 0.0;
        for (long long q = 0; q < w; ++q) { f += hl[q]; l += hl[steps - 1 - q]; }
        st->loss_first = f / (double)w;
        st->loss_last = l / (double)w;
        st->steps = steps;
        st->seconds = std::chrono::duration<double>(t1 - t0).count();
        st->samples_per_second = (double)(steps * nb) / std::max(1e-9, st->seconds);
        st->kernel_launches_per_step = launches;
    }
    return MPF_OK;
}

namespace {
int surrogate_eval(mpf_surrogate* s, int64_t n, const float* inputs, float* out, int hold)
{
    if (!s || n < 0 || (n > 0 && (!inputs || !out))) return fail(MPF_BAD_INPUT, "mpf_surrogate_eval: bad argument");
    if (n == 0) return MPF_OK;
    cudaError_t e = set_smem_attrs();
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_eval: attributes");
    Buffers mem;
    float* x = mem.f((size_t)n * 4);
    float* y = mem.f((size_t)n * kOut);
    unsigned* err = mem.any<unsigned>(sizeof(unsigned));
    if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_eval");
    e = cudaMemcpy(x, inputs, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_eval");
    const long long tiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<long long>((tiles + kWG - 1) / kWG, sm_count());
    k_eval<<<grid, kThreads, kSmemBytes>>>(s->spec, s->packed, x, n, y, err, hold);
    e = cudaGetLastError();
    unsigned herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(out, y, (size_t)n * kOut * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_eval");
    if (herr) return fail(MPF_DEVICE_TIMEOUT, "mpf_surrogate_eval: a tensor-core wait ran out");
    return MPF_OK;
}
}  // namespace

int mpf_surrogate_eval(mpf_surrogate* s, int64_t n, const float* inputs, float* out)
{
    return surrogate_eval(s, n, inputs, out, 0);
}

// Test of the bounded tensor-core wait (no reference counterpart): the same
// evaluation with the MMAs withheld, so that each warpgroup's first
// completion wait runs out after its limit (1 s).  Nothing is left in flight
// (nothing was issued), TMEM is released as usual, and the call returns
// MPF_DEVICE_TIMEOUT with the context still usable.
extern "C" int mpf_internal_surrogate_wait_test(mpf_surrogate* s, int64_t n, const float* inputs, float* out)
{
    return surrogate_eval(s, n, inputs, out, 1);
}

int mpf_surrogate_propagate(mpf_surrogate* s, const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p,
                            const mpf_surrogate_prop_params* sp, int64_t n, const double* launch, int64_t* steps,
                            double* final_rec, uint8_t* flags, float* drift, mpf_surrogate_prop_stats* st)
{
    if (!s || !o || !c || !p || !sp || n < 0 || (n > 0 && (!launch || !steps || !flags)))
        return fail(MPF_BAD_INPUT, "mpf_surrogate_propagate: bad argument");
    if (o->tree.vel)
        return fail(MPF_BAD_INPUT, "mpf_surrogate_propagate: the surrogate has no velocity field; the octree carries one");
    if (p->nplanes != 0 || p->jacobian || p->exact || p->nsteps == 0 || (p->order != 1 && p->order != 2) || p->stop < 0 ||
        p->stop > 6 || !(p->length > 0.0) || !(sp->tolerance >= 0.0) || sp->check_every < 1)
        return fail(MPF_BAD_INPUT, "mpf_surrogate_propagate: unsupported parameters (surfaces, Jacobian and exact mode are "
                                   "plain-path features)");
    if (n == 0) return MPF_OK;
    cudaError_t e = set_smem_attrs();
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_propagate: attributes");
    mpf::PropParams P;
    std::memset(&P, 0, sizeof(P));
    P.length = p->length;
    P.stop_ref = p->stop_value;
    for (int q = 0; q < 3; ++q) P.ki[q] = p->plane_normal[q];
    P.max_steps = (p->max_steps > 0) ? p->max_steps : 100000000ll;
    P.nsteps = p->nsteps;
    P.order = p->order;
    P.stop_kind = p->stop;
    const mpf::DevCosmo C = dev_cosmo(c);
    Buffers mem;
    double* dl = mem.any<double>((size_t)n * 6 * sizeof(double));
    long long* ds = mem.any<long long>((size_t)n * sizeof(long long));
    double* df = final_rec ? mem.any<double>((size_t)n * MPF_PHOTON_FIELDS * sizeof(double)) : nullptr;
    unsigned char* dflag = mem.any<unsigned char>((size_t)n);
    float* ddrift = mem.any<float>((size_t)n * sizeof(float));
    unsigned long long* dcnt = mem.any<unsigned long long>(4 * sizeof(unsigned long long));
    unsigned* dstatus = mem.any<unsigned>(2 * sizeof(unsigned));
    if (mem.err != cudaSuccess) return cuda_fail(mem.err, "mpf_surrogate_propagate");
    e = cudaMemcpy(dl, launch, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dcnt, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(dstatus, 0, 2 * sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "mpf_surrogate_propagate");
    SurrOut O{(long long*)ds, df, dflag, ddrift, dcnt, dstatus};
    const unsigned grid = (unsigned)std::min<long long>(sm_count(), ((n + 127) / 128 + kWG - 1) / kWG);
    cudaEvent_t ev[4];
    for (auto& x : ev) cudaEventCreate(&x);
    cudaEventRecord(ev[0]);
    if (p->order == 1)
        k_propagate_surrogate<1><<<grid, kThreads, kSmemBytes>>>(o->tree, C, P, s->spec, s->packed, dl, n, O, dcnt + 2, dstatus + 1,
                                                               sp->tolerance, sp->check_every);
    else
        k_propagate_surrogate<2><<<grid, kThreads, kSmemBytes>>>(o->tree, C, P, s->spec, s->packed, dl, n, O, dcnt + 2, dstatus + 1,
                                                               sp->tolerance, sp->check_every);
    e = cudaGetLastError();
    cudaEventRecord(ev[1]);
    unsigned long long hc[4] = {0, 0, 0, 0};
    unsigned hs[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hs, dstatus, sizeof(hs), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(steps, ds, (size_t)n * sizeof(int64_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(flags, dflag, (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && drift) e = cudaMemcpy(drift, ddrift, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && final_rec)
        e = cudaMemcpy(final_rec, df, (size_t)n * MPF_PHOTON_FIELDS * sizeof(double), cudaMemcpyDeviceToHost);
    float ms_s = 0.f, ms_f = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms_s, ev[0], ev[1]);
    if (e != cudaSuccess) {
        for (auto& x : ev) cudaEventDestroy(x);
        return cuda_fail(e, "mpf_surrogate_propagate");
    }
    if (hs[1]) {
        for (auto& x : ev) cudaEventDestroy(x);
        return fail(MPF_DEVICE_TIMEOUT, "mpf_surrogate_propagate: a tensor-core wait ran out");
    }
    // fallback: flagged photons re-run on the plain octree path
    long long fb = 0, fb_steps = 0;
    if (sp->fallback) {
        std::vector<long long> idx;
        for (int64_t q = 0; q < n; ++q)
            if (flags[q] & 1u) idx.push_back(q);
        fb = (long long)idx.size();
        if (fb > 0) {
            std::vector<double> sub((size_t)fb * 6);
            for (long long q = 0; q < fb; ++q)
                for (int r = 0; r < 6; ++r) sub[q * 6 + r] = launch[idx[q] * 6 + r];
            std::vector<int64_t> fsteps((size_t)fb);
            std::vector<double> frec(final_rec ? (size_t)fb * MPF_PHOTON_FIELDS : 0);
            mpf_params pp = *p;
            pp.exact = 0;
            cudaEventRecord(ev[2]);
            const int rc = mpf_propagate(o, c, &pp, fb, sub.data(), fsteps.data(), final_rec ? frec.data() : nullptr, nullptr);
            cudaEventRecord(ev[3]);
            cudaEventSynchronize(ev[3]);
            cudaEventElapsedTime(&ms_f, ev[2], ev[3]);
            if (rc < 0) {
                for (auto& x : ev) cudaEventDestroy(x);
                return rc;
            }
            for (long long q = 0; q < fb; ++q) {
                steps[idx[q]] = fsteps[q];
                fb_steps += fsteps[q] - 1;
                if (final_rec) std::memcpy(final_rec + idx[q] * MPF_PHOTON_FIELDS, frec.data() + q * MPF_PHOTON_FIELDS,
                                           MPF_PHOTON_FIELDS * sizeof(double));
            }
        }
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (st) {
        st->photon_steps = (int64_t)hc[0];
        st->flagged_photons = (int64_t)hc[1];
        st->fallback_photons = fb;
        st->fallback_steps = fb_steps;
        st->surrogate_seconds = ms_s * 1e-3;
        st->fallback_seconds = ms_f * 1e-3;
    }
    return (hs[0] & 1u) ? MPF_WARN_MAX_STEPS : MPF_OK;
}

}  // extern "C"
