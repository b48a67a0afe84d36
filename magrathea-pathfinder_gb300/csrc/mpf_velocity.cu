// Velocity field of the cone octree (the reference built with -DVELOCITYFIELD):
// the per-cell velocity slots (src/gravity2.h:45), their deposit from
// particles with CIC or TSC weights at every level of the octree
// (Hmaps::CreateOctreeVelocityWithCIC / WithTSC, src/hmaps.h:439-485,
// 501-550), the zeroed masses before and the mass normalisation and parent
// fill after (src/hmaps.cpp:396, 424-441).  Must be compiled with
// -fmad=false: the weights are the reference's float64 expressions.
//
// The deposit reproduces the reference's accumulation order.  A cell's
// float accumulators (its rho and velocity slots) take, one after another,
// rho += w and v += v_p * w (float += double: the sum is formed in float64
// and rounded to float) for its particles in the order a single thread
// visits them (particle, then vertex).  On the device: every (particle,
// level, vertex) whose cell exists becomes a pair (cell, particle << 5 |
// vertex), the pairs are stably sorted by cell (LSD radix, 4-bit digits,
// block-level ranking in shared memory),
// one thread per pair forms its float64 addends (w, v_p w), and one thread
// per cell adds its run of addends to the float accumulators in order.  The
// result is
// deterministic and bit-identical to the reference run on one thread; the
// reference's own multithreaded loop (Utility::parallelize, src/utility.h:
// 127-147) adds to shared cells without atomics, so its sums vary with the
// thread interleaving.
#include <algorithm>
#include <cstring>
#include <vector>

#include "mpf_internal.h"

namespace mpf {
namespace {

constexpr int kSortThreads = 256;             // radix-sort block
constexpr int kSortItems = 8;                 // keys per thread
constexpr int kSortTile = kSortThreads * kSortItems;   // keys per block and pass
constexpr long long kVelChunk = 1ll << 19;    // particles per pass (payload: particle << 5 | vertex)

__device__ __forceinline__ int rec_level(const DevTree& T, int cell)
{
    return __ldg(reinterpret_cast<const int*>(T.stencil + 8 * (size_t)cell) + 27) & 255;
}
__device__ __forceinline__ int rec_parent(const DevTree& T, int cell)
{
    return __ldg(reinterpret_cast<const int*>(T.stencil + 8 * (size_t)cell) + 30);
}

// Offset of vertex v along each axis: CIC loops iz, iy, ix over {-1, 1}
// (hmaps.h:462-464), TSC over {-1, 0, 1} (hmaps.h:525-530), ix fastest.
__device__ __forceinline__ void vertex_offsets(int scheme, int v, int* o)
{
    if (scheme == 1) {
        o[0] = 2 * (v & 1) - 1;
        o[1] = 2 * ((v >> 1) & 1) - 1;
        o[2] = 2 * ((v >> 2) & 1) - 1;
    } else {
        o[0] = v % 3 - 1;
        o[1] = (v / 3) % 3 - 1;
        o[2] = v / 9 - 1;
    }
}

// One axis's factor of the weight of a particle at coordinate x on the level-L
// cell whose integer coordinate along that axis is c, reached with offset o
// (the vertex cell's centre is the cell's own).  CIC: 1 - |x - centre| /
// extent (hmaps.h:472); TSC: the quadratic weight of |centre - x| / cell
// (hmaps.h:539-545; the cell size is a power of two, so dividing by it is
// the exact product with its inverse).  The weight is the product of the
// three factors, x then y then z, as the reference multiplies them.
__device__ __forceinline__ double axis_factor(int scheme, int L, float x, uint64_t c, int o)
{
    const double cen = coord_center(L, c);
    const double inv = pow2(L - kLevelShift);   // 1 / (EXTENT / 2^L), exact
    if (scheme == 1) return __dsub_rn(1.0, __dmul_rn(fabs(__dsub_rn((double)x, cen)), inv));
    const double dist = fabs(__dmul_rn(__dsub_rn(cen, (double)x), inv));
    const int a = abs(o);
    const double t1 = __dmul_rn(__dmul_rn(__dmul_rn((double)a, 0.5), __dsub_rn(1.5, dist)), __dsub_rn(1.5, dist));
    const double t2 = __dmul_rn((double)(1 - a), __dsub_rn(0.75, __dmul_rn(dist, dist)));
    return __dadd_rn(t1, t2);
}

// pairs per particle: pass 0 counts them (cnt[i]) and writes the particle's
// axis factors per level (axw[(i * nlev + level - lmin) * 9 + 3 * axis +
// offset + 1]); pass 1 writes the pairs at off[i] as (cell, particle << 5 |
// vertex), in the order (level, vertex)
__global__ void k_dep_pairs(DevTree T, int scheme, int lmin, int lmax, const float* __restrict__ pos, long long n,
                            int* cnt, const int* __restrict__ off, unsigned* key, unsigned* pay, double* axw)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const int nv = (scheme == 1) ? 8 : 27;
    int k = 0;
    const long long base = off ? off[i] : 0;
    for (int L = lmin; L <= lmax; ++L) {
        // the level-L cells with the exact key of each vertex (hmaps.h:466-470,
        // 532-536): the vertex is the particle's float position plus (CIC) half a
        // cell or (TSC) one cell times the offset, in float64; its integer
        // coordinates per axis and offset are formed once per level
        const double half = half_cell(L);
        const double step = (scheme == 1) ? half : __dmul_rn(2.0, half);
        uint64_t c[3][3];
        for (int d = 0; d < 3; ++d)
            for (int o = -1; o <= 1; ++o)
                c[d][o + 1] = (scheme == 1 && o == 0) ? 0ull : axis_coord(L, __dadd_rn((double)p[d], __dmul_rn(step, (double)o)));
        if (!off) {
            double* f = axw + ((long long)i * (lmax - lmin + 1) + (L - lmin)) * 9;
            for (int d = 0; d < 3; ++d)
                for (int o = -1; o <= 1; ++o)
                    f[3 * d + o + 1] = (scheme == 1 && o == 0) ? 0.0 : axis_factor(scheme, L, p[d], c[d][o + 1], o);
        }
        for (int v = 0; v < nv; ++v) {
            int ov[3];
            vertex_offsets(scheme, v, ov);
            const Found f = find_cell(T, L, c[0][ov[0] + 1], c[1][ov[1] + 1], c[2][ov[2] + 1]);
            if (f.cell < 0 || f.level != L) continue;
            if (off) {
                key[base + k] = (unsigned)f.cell;
                pay[base + k] = ((unsigned)i << 5) | (unsigned)v;
            }
            ++k;
        }
    }
    if (!off) cnt[i] = k;
}

// Stable LSD radix sort of (key, pay) by key, 4-bit digits.  Per pass: each
// block of kSortThreads threads takes a tile of kSortTile consecutive pairs
// (thread t the kSortItems pairs from t * kSortItems); k_sort_hist writes the
// tile's digit counts (digit-major, tile-minor, so that their exclusive scan
// gives every (digit, tile) its stable global start); k_sort_scatter ranks
// the tile's keys by digit in shared memory (an exclusive scan over the
// digit-major array of per-thread counts keeps the tile's order within a
// digit) and writes each digit's run to consecutive global addresses.
__device__ __forceinline__ void sort_load(long long m, long long tile, const unsigned* __restrict__ key, unsigned* k, int* valid)
{
    const long long j0 = tile * kSortTile + (long long)threadIdx.x * kSortItems;
#pragma unroll
    for (int q = 0; q < kSortItems; ++q) {
        const long long j = j0 + q;
        valid[q] = j < m;
        k[q] = valid[q] ? key[j] : 0u;
    }
}

__global__ void __launch_bounds__(kSortThreads) k_sort_hist(long long m, const unsigned* __restrict__ key, int shift,
                                                            int* hist, long long ntiles)
{
    __shared__ int h[16];
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    unsigned k[kSortItems];
    int valid[kSortItems];
    sort_load(m, blockIdx.x, key, k, valid);
#pragma unroll
    for (int q = 0; q < kSortItems; ++q)
        if (valid[q]) atomicAdd(&h[(k[q] >> shift) & 15u], 1);
    __syncthreads();
    if (threadIdx.x < 16) hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(long long m, const unsigned* __restrict__ key,
                                                               const unsigned* __restrict__ pay, int shift,
                                                               const int* __restrict__ off, long long ntiles,
                                                               unsigned* key2, unsigned* pay2)
{
    __shared__ int sc[16 * kSortThreads];   // digit-major: sc[d * kSortThreads + t]
    __shared__ unsigned sk[kSortTile], sp[kSortTile];
    __shared__ int wsum[kSortThreads / 32];
    __shared__ long long goff[16];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long tile = blockIdx.x;
    unsigned k[kSortItems], pv[kSortItems];
    int valid[kSortItems];
    sort_load(m, tile, key, k, valid);
    const long long j0 = tile * kSortTile + (long long)t * kSortItems;
#pragma unroll
    for (int q = 0; q < kSortItems; ++q) pv[q] = valid[q] ? pay[j0 + q] : 0u;
    int c[16];
#pragma unroll
    for (int d = 0; d < 16; ++d) c[d] = 0;
#pragma unroll
    for (int q = 0; q < kSortItems; ++q)
        if (valid[q]) ++c[(k[q] >> shift) & 15u];
#pragma unroll
    for (int d = 0; d < 16; ++d) sc[d * kSortThreads + t] = c[d];
    if (t < 16) goff[t] = off[t * ntiles + tile];
    __syncthreads();
    // exclusive scan of the flat array: thread t scans its 16 consecutive entries,
    // then the threads' totals are scanned across the block
    int loc[16], run = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        loc[q] = run;
        run += sc[t * 16 + q];
    }
    int incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    const int excl = before + incl - run;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) sc[t * 16 + q] = excl + loc[q];
    __syncthreads();
    // place this thread's keys in the tile, in order within each digit
    int base[16];
#pragma unroll
    for (int d = 0; d < 16; ++d) base[d] = sc[d * kSortThreads + t];
#pragma unroll
    for (int q = 0; q < kSortItems; ++q) {
        if (!valid[q]) continue;
        const int d = (k[q] >> shift) & 15u;
        const int at = base[d]++;
        sk[at] = k[q];
        sp[at] = pv[q];
    }
    __syncthreads();
    const long long rem = m - tile * kSortTile;
    const int count = (int)(rem < kSortTile ? rem : kSortTile);
    for (int i = t; i < count; i += kSortThreads) {
        const unsigned kk = sk[i];
        const int d = (kk >> shift) & 15u;
        const long long dst = goff[d] + (i - sc[d * kSortThreads]);
        key2[dst] = kk;
        pay2[dst] = sp[i];
    }
}

// the float64 addends of pair (particle << 5 | vertex) on a level-L cell: w
// (the product of the particle's three axis factors) and v_p w
__device__ __forceinline__ void pair_addends(int scheme, int L, int lmin, int nlev, const double* __restrict__ axw,
                                             const float* __restrict__ pv, unsigned pj, double* a)
{
    const long long i = pj >> 5;
    int o[3];
    vertex_offsets(scheme, (int)(pj & 31u), o);
    const double* f = axw + (i * nlev + (L - lmin)) * 9;
    const double w = __dmul_rn(__dmul_rn(__ldg(f + o[0] + 1), __ldg(f + 3 + o[1] + 1)), __ldg(f + 6 + o[2] + 1));
    a[0] = w;
    a[1] = __dmul_rn((double)__ldg(pv + 3 * i), w);
    a[2] = __dmul_rn((double)__ldg(pv + 3 * i + 1), w);
    a[3] = __dmul_rn((double)__ldg(pv + 3 * i + 2), w);
}

// run starts of the sorted pairs: flag[j] = 1 where a cell's run begins
__global__ void k_dep_run_flags(long long m, const unsigned* __restrict__ key, int* flag)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) flag[j] = (j == 0 || key[j] != key[j - 1]) ? 1 : 0;
}
__global__ void k_dep_run_list(long long m, const unsigned* __restrict__ key, const int* __restrict__ idx, unsigned* runs)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m && (j == 0 || key[j] != key[j - 1])) runs[idx[j]] = (unsigned)j;
}

// The float64 addends of every sorted pair, one thread per pair (the
// weights' float64 arithmetic, balanced over the whole grid).
__global__ void k_dep_addends(DevTree T, int scheme, int lmin, int nlev, const double* __restrict__ axw,
                              const float* __restrict__ pv, long long m, const unsigned* __restrict__ key,
                              const unsigned* __restrict__ pay, double2* add)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    double a[4];
    pair_addends(scheme, rec_level(T, (int)key[j]), lmin, nlev, axw, pv, pay[j], a);
    add[2 * j] = make_double2(a[0], a[1]);
    add[2 * j + 1] = make_double2(a[2], a[3]);
}

// Length class of each run (1 + floor(log2(length)), at most 15) as a sort
// key, with the run's start as its payload: sorted by class, the runs a warp
// takes have about the same length.
__global__ void k_dep_run_class(long long m, const unsigned* __restrict__ runs, long long nruns, unsigned* ckey,
                                unsigned* cpay)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    const long long len = ((r + 1 < nruns) ? (long long)runs[r + 1] : m) - (long long)runs[r];
    const int cls = 64 - __clzll((unsigned long long)len);
    ckey[r] = (unsigned)min(cls, 15);
    cpay[r] = runs[r];
}

// One thread per cell run (the runs in length-class order): the reference's
// sequential float += in order, four independent chains (rho, vx, vy, vz).
__global__ void k_dep_accumulate(const unsigned* __restrict__ key, float4* scal, float4* vel, long long m,
                                 const double2* __restrict__ add, const unsigned* __restrict__ starts, long long nruns)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    const long long j0 = starts[r];
    const int cell = (int)key[j0];
    long long j1 = j0 + 1;
    while (j1 < m && key[j1] == (unsigned)cell) ++j1;
    const float4 u0 = vel[cell];
    float acc[4] = {scal[cell].x, u0.x, u0.y, u0.z};
    for (long long j = j0; j < j1; ++j) {
        const double2 a01 = add[2 * j], a23 = add[2 * j + 1];
        acc[0] = __double2float_rn(__dadd_rn((double)acc[0], a01.x));
        acc[1] = __double2float_rn(__dadd_rn((double)acc[1], a01.y));
        acc[2] = __double2float_rn(__dadd_rn((double)acc[2], a23.x));
        acc[3] = __double2float_rn(__dadd_rn((double)acc[3], a23.y));
    }
    scal[cell].x = acc[0];
    vel[cell] = make_float4(acc[1], acc[2], acc[3], u0.w);
}

__global__ void k_dep_begin(long long n, float4* scal, float4* vel)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    scal[i].x = 0.f;
    vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// v /= mass, a zero mass read as 1 (hmaps.cpp:425-431)
__global__ void k_dep_normalise(long long n, const float4* __restrict__ scal, float4* vel)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double mass = (double)scal[i].x;
    mass = __dadd_rn(mass, (double)(mass == 0.0));
    float4 u = vel[i];
    u.x = __double2float_rn(__ddiv_rn((double)u.x, mass));
    u.y = __double2float_rn(__ddiv_rn((double)u.y, mass));
    u.z = __double2float_rn(__ddiv_rn((double)u.z, mass));
    vel[i] = u;
}

// std::isnormal of a float: neither zero, subnormal, infinite nor NaN
__device__ __forceinline__ bool normal_f(float x)
{
    const unsigned b = __float_as_uint(x) & 0x7fffffffu;
    return b >= 0x00800000u && b < 0x7f800000u;
}

// cells of level L whose mass is not normal take their parent's velocity
// (hmaps.cpp:433-441); the parent, one level up, is final already
__global__ void k_dep_from_parent(DevTree T, long long n, int L, const float4* __restrict__ scal, float4* vel)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (rec_level(T, (int)i) != L || normal_f(scal[i].x)) return;
    const int par = rec_parent(T, (int)i);
    if (par < 0) return;
    const float4 pu = vel[par];
    float4 u = vel[i];
    u.x = pu.x; u.y = pu.y; u.z = pu.z;
    vel[i] = u;
}

__global__ void k_vel_set(long long n, const float* __restrict__ v3, const float* __restrict__ rho, float4* scal, float4* vel)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vel[i] = make_float4(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2], 0.f);
    if (rho) scal[i].x = rho[i];
}

__global__ void k_vel_get(long long n, const float4* __restrict__ scal, const float4* __restrict__ vel, float* v3, float* rho)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (v3) {
        const float4 u = vel ? vel[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        v3[3 * i] = u.x; v3[3 * i + 1] = u.y; v3[3 * i + 2] = u.z;
    }
    if (rho) rho[i] = scal[i].x;
}

inline unsigned blocks(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// device buffer freed on scope exit
struct DevMem {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevMem() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t b)
    {
        bytes = b ? b : 1;
        return cudaMalloc(&p, bytes);
    }
    // at least b bytes, keeping the buffer when it is large enough
    cudaError_t reserve(size_t b)
    {
        if (p && bytes >= b) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        return alloc(b);
    }
    template <class T> T* as() const { return (T*)p; }
};

cudaError_t ensure_velocity(mpf_octree* o)
{
    if (o->vel) return cudaSuccess;
    cudaError_t e = cudaMalloc(&o->vel, (size_t)o->n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(o->vel, 0, (size_t)o->n * sizeof(float4));
    if (e != cudaSuccess) {
        if (o->vel) cudaFree(o->vel);
        o->vel = nullptr;
        return e;
    }
    o->tree.vel = o->vel;
    return cudaSuccess;
}

// Scratch of one deposit call, grown as its passes need: per-particle pair
// counts, the pairs and their sorted copies, the radix histograms.
struct DepScratch {
    DevMem cnt, key, pay, key2, pay2, hist, add, runs, axw;
    long long pairs = 0;   // pairs of all passes (reported by the bench)
};

// one pass over particles [0, n) of a chunk on the device, on stream s
cudaError_t deposit_chunk(mpf_octree* o, int scheme, const float* d_pos, const float* d_vel, long long n, DepScratch& S,
                          cudaStream_t s)
{
    const DevTree& T = o->tree;
    const int nlev = o->level_max - o->level_min + 1;
    cudaError_t e = S.cnt.reserve((size_t)(n + 1) * sizeof(int));
    if (e == cudaSuccess) e = S.axw.reserve((size_t)n * nlev * 9 * sizeof(double));
    if (e != cudaSuccess) return e;
    int* cnt = S.cnt.as<int>();
    double* axw = S.axw.as<double>();
    k_dep_pairs<<<blocks(n, 128), 128, 0, s>>>(T, scheme, o->level_min, o->level_max, d_pos, n, cnt, nullptr, nullptr,
                                                nullptr, axw);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(cnt + n, 0, sizeof(int), s)) != cudaSuccess) return e;
    const long long m = exclusive_scan(cnt, n + 1, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (m <= 0) return cudaSuccess;
    S.pairs += m;
    const long long ntiles = (m + kSortTile - 1) / kSortTile;
    // key buffers hold m + 1 entries: after the sort the spare one holds the run flags and their scan total
    if ((e = S.key.reserve((size_t)(m + 1) * 4)) != cudaSuccess || (e = S.pay.reserve((size_t)m * 4)) != cudaSuccess ||
        (e = S.key2.reserve((size_t)(m + 1) * 4)) != cudaSuccess || (e = S.pay2.reserve((size_t)m * 4)) != cudaSuccess ||
        (e = S.hist.reserve((size_t)(16 * ntiles + 1) * sizeof(int))) != cudaSuccess)
        return e;
    unsigned *k1 = S.key.as<unsigned>(), *p1 = S.pay.as<unsigned>(), *k2 = S.key2.as<unsigned>(), *p2 = S.pay2.as<unsigned>();
    int* hist = S.hist.as<int>();
    k_dep_pairs<<<blocks(n, 128), 128, 0, s>>>(T, scheme, o->level_min, o->level_max, d_pos, n, nullptr, cnt, k1, p1,
                                                nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // digits up to the highest bit of the largest cell index
    int bits = 1;
    while (bits < 31 && (1ll << bits) < o->n) ++bits;
    for (int shift = 0; shift < bits; shift += 4) {
        k_sort_hist<<<(unsigned)ntiles, kSortThreads, 0, s>>>(m, k1, shift, hist, ntiles);
        exclusive_scan(hist, 16 * ntiles, s);
        k_sort_scatter<<<(unsigned)ntiles, kSortThreads, 0, s>>>(m, k1, p1, shift, hist, ntiles, k2, p2);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        std::swap(k1, k2);
        std::swap(p1, p2);
    }
    // the runs of equal cells (the sort's spare buffers hold the flags and the list)
    int* flag = reinterpret_cast<int*>(k2);
    unsigned* runs = p2;
    k_dep_run_flags<<<blocks(m, 256), 256, 0, s>>>(m, k1, flag);
    if ((e = cudaMemsetAsync(flag + m, 0, sizeof(int), s)) != cudaSuccess) return e;
    const long long nruns = exclusive_scan(flag, m + 1, s);
    k_dep_run_list<<<blocks(m, 256), 256, 0, s>>>(m, k1, flag, runs);
    if ((e = S.add.reserve((size_t)m * 2 * sizeof(double2))) != cudaSuccess) return e;
    double2* add = S.add.as<double2>();
    k_dep_addends<<<blocks(m, 128), 128, 0, s>>>(T, scheme, o->level_min, nlev, axw, d_vel, m, k1, p1, add);
    // the runs sorted by length class (one radix pass: the class fits a digit)
    if ((e = S.runs.reserve((size_t)nruns * 4 * sizeof(unsigned))) != cudaSuccess) return e;
    unsigned *ck = S.runs.as<unsigned>(), *cp = ck + nruns, *ck2 = cp + nruns, *cp2 = ck2 + nruns;
    k_dep_run_class<<<blocks(nruns, 256), 256, 0, s>>>(m, runs, nruns, ck, cp);
    const long long rtiles = (nruns + kSortTile - 1) / kSortTile;
    k_sort_hist<<<(unsigned)rtiles, kSortThreads, 0, s>>>(nruns, ck, 0, hist, rtiles);
    exclusive_scan(hist, 16 * rtiles, s);
    k_sort_scatter<<<(unsigned)rtiles, kSortThreads, 0, s>>>(nruns, ck, cp, 0, hist, rtiles, ck2, cp2);
    k_dep_accumulate<<<blocks(nruns, 128), 128, 0, s>>>(k1, o->scal, o->vel, m, add, cp2, nruns);
    return cudaGetLastError();
}

// The deposit call: particles from host (copied per pass) or device memory.
int deposit(const char* who, mpf_octree* o, int scheme, long long n, const float* pos, const float* vel, int flags,
            bool on_device, cudaStream_t s)
{
    if (!o || (scheme != 1 && scheme != 2) || n < 0 || (n > 0 && (!pos || !vel)) || (flags & ~3))
        return mpf_internal_set_error(MPF_BAD_INPUT, who);
    if (!(flags & MPF_VELOCITY_BEGIN) && !o->vel)
        return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_velocity_deposit: the octree has no velocity field "
                                                     "(start with MPF_VELOCITY_BEGIN)");
    if (o->n >= (1ll << 31)) return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_velocity_deposit: octree too large");
    cudaError_t e = ensure_velocity(o);
    if (e == cudaSuccess && (flags & MPF_VELOCITY_BEGIN)) {
        k_dep_begin<<<blocks(o->n, 256), 256, 0, s>>>(o->n, o->scal, o->vel);
        e = cudaGetLastError();
    }
    DepScratch S;
    if (e == cudaSuccess && n > 0) {
        // at most kVelChunk particles and about 2^27 pairs per pass (2 GB of sort
        // buffers, 4 GB of float64 addends)
        const long long per = (long long)((scheme == 1) ? 8 : 27) * (o->level_max - o->level_min + 1);
        const long long chunk = std::min<long long>(n, std::max<long long>(1024, std::min<long long>(kVelChunk, (1ll << 27) / per)));
        DevMem dp, dv;
        if (!on_device) {
            e = dp.alloc((size_t)chunk * 3 * sizeof(float));
            if (e == cudaSuccess) e = dv.alloc((size_t)chunk * 3 * sizeof(float));
        }
        for (long long lo = 0; lo < n && e == cudaSuccess; lo += chunk) {
            const long long m = std::min<long long>(chunk, n - lo);
            const float *cp = pos + 3 * lo, *cv = vel + 3 * lo;
            if (!on_device) {
                e = cudaMemcpyAsync(dp.p, cp, (size_t)m * 3 * sizeof(float), cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess) e = cudaMemcpyAsync(dv.p, cv, (size_t)m * 3 * sizeof(float), cudaMemcpyHostToDevice, s);
                cp = dp.as<float>();
                cv = dv.as<float>();
            }
            if (e == cudaSuccess) e = deposit_chunk(o, scheme, cp, cv, m, S, s);
            // the next pass reuses the particle staging and the sort buffers
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    if (e == cudaSuccess && (flags & MPF_VELOCITY_FINISH)) {
        k_dep_normalise<<<blocks(o->n, 256), 256, 0, s>>>(o->n, o->scal, o->vel);
        for (int L = o->level_min + 1; L <= o->level_max; ++L)
            k_dep_from_parent<<<blocks(o->n, 256), 256, 0, s>>>(o->tree, o->n, L, o->scal, o->vel);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mpf_internal_set_error(MPF_CUDA_ERROR, cudaGetErrorString(e));
    o->deposit_pairs = S.pairs;
    return MPF_OK;
}

}  // namespace
}  // namespace mpf

using namespace mpf;

extern "C" {

int mpf_octree_set_velocity(mpf_octree* o, const float* v3, const float* rho)
{
    if (!o) return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_octree_set_velocity: null octree");
    if (!v3) {
        if (rho) return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_octree_set_velocity: rho without velocities");
        if (o->vel) cudaFree(o->vel);
        o->vel = nullptr;
        o->tree.vel = nullptr;
        return MPF_OK;
    }
    const long long n = o->n;
    DevMem dv, dr;
    cudaError_t e = ensure_velocity(o);
    if (e == cudaSuccess) e = dv.alloc((size_t)n * 3 * sizeof(float));
    if (e == cudaSuccess && rho) e = dr.alloc((size_t)n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dv.p, v3, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && rho) e = cudaMemcpy(dr.p, rho, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_vel_set<<<blocks(n, 256), 256>>>(n, dv.as<float>(), rho ? dr.as<float>() : nullptr, o->scal, o->vel);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return mpf_internal_set_error(MPF_CUDA_ERROR, cudaGetErrorString(e));
    return MPF_OK;
}

int mpf_octree_get_velocity(const mpf_octree* o, float* v3, float* rho)
{
    if (!o || (!v3 && !rho)) return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_octree_get_velocity: bad argument");
    const long long n = o->n;
    DevMem dv, dr;
    cudaError_t e = cudaSuccess;
    if (v3) e = dv.alloc((size_t)n * 3 * sizeof(float));
    if (e == cudaSuccess && rho) e = dr.alloc((size_t)n * sizeof(float));
    if (e == cudaSuccess) {
        k_vel_get<<<blocks(n, 256), 256>>>(n, o->scal, o->vel, v3 ? dv.as<float>() : nullptr, rho ? dr.as<float>() : nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && v3) e = cudaMemcpy(v3, dv.p, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && rho) e = cudaMemcpy(rho, dr.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return mpf_internal_set_error(MPF_CUDA_ERROR, cudaGetErrorString(e));
    return o->vel ? MPF_OK : mpf_internal_set_error(MPF_OK, "mpf_octree_get_velocity: the octree has no velocity field");
}

int mpf_velocity_deposit(mpf_octree* o, int scheme, int64_t n, const float* pos, const float* vel, int flags)
{
    return deposit("mpf_velocity_deposit: bad argument", o, scheme, n, pos, vel, flags, false, 0);
}

int mpf_velocity_deposit_device(mpf_octree* o, int scheme, int64_t n, const float* pos_device, const float* vel_device,
                                int flags, void* stream)
{
    return deposit("mpf_velocity_deposit_device: bad argument", o, scheme, n, pos_device, vel_device, flags, true,
                   (cudaStream_t)stream);
}

int mpf_velocity_deposit_pairs(const mpf_octree* o, int64_t* pairs)
{
    if (!o || !pairs) return mpf_internal_set_error(MPF_BAD_INPUT, "mpf_velocity_deposit_pairs: bad argument");
    *pairs = o->deposit_pairs;
    return MPF_OK;
}

}  // extern "C"
