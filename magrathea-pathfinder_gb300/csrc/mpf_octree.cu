// Device octree build from the reference's 48-byte cone records
// (src/input.h:1275-1313 on-disk format; layout of Gravity<float,3> in a
// std::pair with a 128-bit key: key 0-15, dphidt 16, a 20, dphidx 24,
// dphidy 28, dphidz 32, phi 36, rho 40).
//
// All passes run on the GPU:
//   1. unpack records into keys / grad / scal, check the keys are strictly
//      increasing (the reference always saves after update()), level range;
//   2. pick the top level Lt (the coarsest level, or coarser when the dense
//      bounding-box grid at that level would exceed the grid budget);
//   3. level by level from Lt: nodes are the distinct level-l prefixes of the
//      keys of level >= l, in key order; a node with deeper keys gets 8
//      contiguous child slots (exclusive scan), each key's level-(l+1) node is
//      its parent's base + its site, and a key of exactly level l+1 names its
//      node's cell;
//   4. scatter the level-Lt nodes into the dense top grid;
//   5. per cell, its stencil record: the 27 same-level lookups around it with
//      the reference's lookup semantics, resolved once here so that a TSC
//      gather during propagation is one record load plus the payload loads.
#include <cstdio>
#include <vector>

#include "mpf_internal.h"

namespace mpf {

namespace {

constexpr int kScanBlock = 1024;

__global__ void k_scan_block(int* d, int64_t n, int* block_sums)
{
    __shared__ int s[kScanBlock];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const int v = (i < n) ? d[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        const int t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) d[i] = s[threadIdx.x] - v;   // exclusive
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_add(int* d, int64_t n, const int* block_offsets)
{
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) d[i] += block_offsets[blockIdx.x];
}

struct Record48 {
    unsigned long long lo, hi;
    float dphidt, a, dphidx, dphidy, dphidz, phi, rho;
    unsigned pad;
};
static_assert(sizeof(Record48) == 48, "record layout");

__global__ void k_unpack(const Record48* __restrict__ rec, int64_t n, ulonglong2* keys, float4* grad, float4* scal,
                         int* lvl_minmax, unsigned* bad)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Record48 r = rec[i];
    keys[i] = make_ulonglong2(r.hi, r.lo);
    grad[i] = make_float4(r.dphidx, r.dphidy, r.dphidz, r.dphidt);
    const int L = key_level(Key{r.hi, r.lo});
    scal[i] = make_float4(r.rho, r.phi, r.a, __int_as_float(L));
    atomicMin(lvl_minmax, L);
    atomicMax(lvl_minmax + 1, L);
    if (i > 0) {
        const Record48 q = rec[i - 1];
        if (!key_less(Key{q.hi, q.lo}, Key{r.hi, r.lo})) atomicOr(bad, 1u);
    }
}

__device__ __forceinline__ uint64_t key_axis(Key k, int level, int dim)
{
    uint64_t c = 0;
    for (int i = 1; i <= level; ++i) {
        const uint64_t w = (i <= 16) ? k.hi : k.lo;
        const int sh = (i <= 16) ? (64 - 4 * i) : (128 - 4 * i);
        c = (c << 1) | ((w >> (sh + dim)) & 1ull);
    }
    return c;
}

__device__ __forceinline__ int key_site(Key k, int level)
{
    const uint64_t w = (level <= 16) ? k.hi : k.lo;
    const int sh = (level <= 16) ? (64 - 4 * level) : (128 - 4 * level);
    return (int)((w >> sh) & 7ull);
}

__global__ void k_bbox(const ulonglong2* keys, int64_t n, int Lt, int* bb)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Key k{keys[i].x, keys[i].y};
    for (int d = 0; d < 3; ++d) {
        const int c = (int)key_axis(k, Lt, d);
        atomicMin(bb + d, c);
        atomicMax(bb + 3 + d, c);
    }
}

// level-Lt node starts: first key of each distinct Lt prefix
__global__ void k_top_flags(const ulonglong2* keys, int64_t n, int Lt, int* flag)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int f = 1;
    if (i > 0) {
        const Key a{keys[i - 1].x, keys[i - 1].y}, b{keys[i].x, keys[i].y};
        f = 0;
        for (int d = 0; d < 3 && !f; ++d) f = key_axis(a, Lt, d) != key_axis(b, Lt, d);
    }
    flag[i] = f;
}

// after the exclusive scan of flags: node id = scan + flag - 1 (inclusive - 1)
__global__ void k_top_ids(const ulonglong2* keys, const float4* scal, int64_t n, int Lt, const int* flag_scan,
                          const int* flag, int* nodeid, int2* node, int* grid, int gx0, int gy0, int gz0, int gnx, int gny)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = flag_scan[i] + flag[i] - 1;
    nodeid[i] = id;
    if (flag[i]) {
        node[id] = make_int2(-1, -1);
        const Key k{keys[i].x, keys[i].y};
        const long gx = (long)key_axis(k, Lt, 0) - gx0, gy = (long)key_axis(k, Lt, 1) - gy0, gz = (long)key_axis(k, Lt, 2) - gz0;
        grid[(gz * gny + gy) * (long)gnx + gx] = id;
    }
}

__global__ void k_top_cells(const float4* scal, int64_t n, int Lt, const int* nodeid, int2* node, int* cell_node)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (__float_as_int(scal[i].w) == Lt) {
        node[nodeid[i]].y = (int)i;
        cell_node[i] = nodeid[i];
    }
}

// mark level-l nodes that own a deeper key
__global__ void k_mark(const float4* scal, int64_t n, int l, const int* nodeid, int64_t off_l, int* has)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (__float_as_int(scal[i].w) > l) has[nodeid[i] - off_l] = 1;
}

__global__ void k_children(int64_t cnt_l, int64_t off_l, int64_t off_next, const int* has, const int* scan, int2* node,
                           int2* next)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cnt_l) return;
    if (has[j]) {
        const int base = (int)(off_next + 8 * (int64_t)scan[j]);
        node[off_l + j].x = base;
        for (int s = 0; s < 8; ++s) next[base - off_next + s] = make_int2(-1, -1);
    }
}

// a key's level-(l+1) node: its level-l node's first child + its site
// (ids are global; `cur` holds level l from global id off_l, `next` level l+1
// from global id off_next)
__global__ void k_descend(const ulonglong2* keys, const float4* scal, int64_t n, int l, const int* nodeid, int* nodeid_next,
                          const int2* cur, int64_t off_l, int2* next, int64_t off_next, int* cell_node)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int L = __float_as_int(scal[i].w);
    if (L <= l) { nodeid_next[i] = -1; return; }
    const Key k{keys[i].x, keys[i].y};
    const int id = cur[nodeid[i] - off_l].x + key_site(k, l + 1);
    nodeid_next[i] = id;
    if (L == l + 1) {
        next[id - off_next].y = (int)i;
        cell_node[i] = id;
    }
}

// Stencil record of each cell (layout in mpf_device.cuh).
__global__ void k_stencil(DevTree T, const int* cell_node, int4* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.n) return;
    const Key k{T.keys[i].x, T.keys[i].y};
    const int L = __float_as_int(T.scal[i].w);
    const uint64_t cx = key_axis(k, L, 0), cy = key_axis(k, L, 1), cz = key_axis(k, L, 2);
    const uint64_t mask = (L >= 32) ? 0xffffffffull : ((1ull << L) - 1ull);
    int e[32];
    unsigned exact = 0;
    int j = 0;
    for (int ix = -1; ix <= 1; ++ix)
        for (int iy = -1; iy <= 1; ++iy)
            for (int iz = -1; iz <= 1; ++iz, ++j) {
                const Found f = find_cell(T, L, (cx + (uint64_t)(int64_t)ix) & mask, (cy + (uint64_t)(int64_t)iy) & mask,
                                          (cz + (uint64_t)(int64_t)iz) & mask);
                e[j] = f.cell;
                if (f.cell >= 0 && f.level == L) exact |= 1u << j;
            }
    const int nd = cell_node[i];
    e[27] = L | ((T.node[nd].x >= 0) ? 256 : 0);
    e[28] = (int)exact;
    e[29] = nd;
    // the parent cell (one level up), for restarts at coarser levels
    int parent = -1;
    if (L - 1 >= T.Lt) {
        const Found f = find_cell(T, L - 1, cx >> 1, cy >> 1, cz >> 1);
        if (f.cell >= 0 && f.level == L - 1) parent = f.cell;
    }
    e[30] = parent;
    e[31] = 0;
    int4* o = out + 8 * i;
    for (int q = 0; q < 8; ++q) o[q] = make_int4(e[4 * q], e[4 * q + 1], e[4 * q + 2], e[4 * q + 3]);
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int64_t exclusive_scan(int* d, int64_t n, cudaStream_t stream)
{
    if (n <= 0) return 0;
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    int* sums = nullptr;
    cudaMallocAsync(&sums, (size_t)(nb + 1) * sizeof(int), stream);
    k_scan_block<<<(unsigned)nb, kScanBlock, 0, stream>>>(d, n, sums);
    int64_t total;
    if (nb > 1) {
        total = exclusive_scan(sums, nb, stream);
        k_scan_add<<<(unsigned)nb, kScanBlock, 0, stream>>>(d, n, sums);
    } else {
        int s = 0;
        cudaMemcpyAsync(&s, sums, sizeof(int), cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        total = s;
    }
    cudaFreeAsync(sums, stream);
    return total;
}

}  // namespace mpf

using namespace mpf;

// Budget of the dense top grid, in entries (4 bytes each).
static const int64_t kGridBudget = 1ll << 28;

extern "C" int mpf_internal_octree_build(const void* records, int64_t n, int on_device, cudaStream_t stream,
                                         mpf_octree** out, char* err, int errlen)
{
    auto fail = [&](const char* msg, int code) {
        if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", msg);
        return code;
    };
    if (n <= 0 || n >= (1ll << 31) - 2) return fail("cell count out of range", -1);
    mpf_octree* o = new mpf_octree();
    cudaGetDevice(&o->device);
    o->n = n;
    std::vector<void*> temps;
    auto release = [&](bool all) {
        for (void* t : temps) cudaFree(t);
        temps.clear();
        if (all) {
            cudaFree(o->keys); cudaFree(o->grad); cudaFree(o->scal); cudaFree(o->node); cudaFree(o->grid);
            cudaFree(o->stencil);
            delete o;
        }
    };
    auto dalloc = [&](void** p, size_t bytes, bool temp) {
        if (cudaMalloc(p, bytes) != cudaSuccess) return false;
        if (temp) temps.push_back(*p);
        return true;
    };
    const Record48* drec = (const Record48*)records;
    if (!on_device) {
        void* d = nullptr;
        if (!dalloc(&d, (size_t)n * 48, true)) { release(true); return fail("out of device memory", -2); }
        cudaMemcpyAsync(d, records, (size_t)n * 48, cudaMemcpyHostToDevice, stream);
        drec = (const Record48*)d;
    }
    int* dscratch = nullptr;   // [0..1] level min/max, [2..7] bbox, [8] unsorted flag
    if (!dalloc((void**)&o->keys, (size_t)n * sizeof(ulonglong2), false) || !dalloc((void**)&o->grad, (size_t)n * sizeof(float4), false) ||
        !dalloc((void**)&o->scal, (size_t)n * sizeof(float4), false) || !dalloc((void**)&dscratch, 16 * sizeof(int), true)) {
        release(true);
        return fail("out of device memory", -2);
    }
    int init[16] = {1 << 30, -1, 1 << 30, 1 << 30, 1 << 30, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0};
    cudaMemcpyAsync(dscratch, init, sizeof(init), cudaMemcpyHostToDevice, stream);
    k_unpack<<<blocks(n, 256), 256, 0, stream>>>(drec, n, o->keys, o->grad, o->scal, dscratch, (unsigned*)(dscratch + 8));
    int h[16];
    cudaMemcpyAsync(h, dscratch, sizeof(h), cudaMemcpyDeviceToHost, stream);
    cudaError_t ce = cudaStreamSynchronize(stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) { release(true); return fail(cudaGetErrorString(ce), -3); }
    if (h[8]) { release(true); return fail("records are not strictly increasing by key", -4); }
    o->level_min = h[0];
    o->level_max = h[1];
    // top level and its bounding box
    int Lt = o->level_min;
    int bb[6];
    for (;;) {
        int ib[6] = {1 << 30, 1 << 30, 1 << 30, -1, -1, -1};
        cudaMemcpyAsync(dscratch + 2, ib, sizeof(ib), cudaMemcpyHostToDevice, stream);
        k_bbox<<<blocks(n, 256), 256, 0, stream>>>(o->keys, n, Lt, dscratch + 2);
        cudaMemcpyAsync(bb, dscratch + 2, sizeof(bb), cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        const int64_t vol = (int64_t)(bb[3] - bb[0] + 1) * (bb[4] - bb[1] + 1) * (bb[5] - bb[2] + 1);
        if (vol <= kGridBudget || Lt == 0) break;
        --Lt;
    }
    const int gnx = bb[3] - bb[0] + 1, gny = bb[4] - bb[1] + 1, gnz = bb[5] - bb[2] + 1;
    const int64_t gsz = (int64_t)gnx * gny * gnz;
    int *flag = nullptr, *fscan = nullptr, *nid = nullptr, *nid2 = nullptr, *cell_node = nullptr;
    if (!dalloc((void**)&o->grid, (size_t)gsz * sizeof(int), false) || !dalloc((void**)&flag, (size_t)n * sizeof(int), true) ||
        !dalloc((void**)&cell_node, (size_t)n * sizeof(int), true) ||
        !dalloc((void**)&fscan, (size_t)n * sizeof(int), true) || !dalloc((void**)&nid, (size_t)n * sizeof(int), true) ||
        !dalloc((void**)&nid2, (size_t)n * sizeof(int), true)) {
        release(true);
        return fail("out of device memory", -2);
    }
    cudaMemsetAsync(o->grid, 0xff, (size_t)gsz * sizeof(int), stream);
    k_top_flags<<<blocks(n, 256), 256, 0, stream>>>(o->keys, n, Lt, flag);
    cudaMemcpyAsync(fscan, flag, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, stream);
    const int64_t cnt_top = exclusive_scan(fscan, n, stream);

    // level chunks, addressed by global node id during the build
    std::vector<int2*> chunks;
    std::vector<int64_t> counts, offsets;
    int2* top = nullptr;
    if (!dalloc((void**)&top, (size_t)cnt_top * sizeof(int2), true)) { release(true); return fail("out of device memory", -2); }
    k_top_ids<<<blocks(n, 256), 256, 0, stream>>>(o->keys, o->scal, n, Lt, fscan, flag, nid, top, o->grid, bb[0], bb[1], bb[2],
                                                  gnx, gny);
    k_top_cells<<<blocks(n, 256), 256, 0, stream>>>(o->scal, n, Lt, nid, top, cell_node);
    chunks.push_back(top);
    counts.push_back(cnt_top);
    offsets.push_back(0);
    int64_t total = cnt_top;
    for (int l = Lt; l < o->level_max; ++l) {
        const int64_t cnt = counts.back(), off = offsets.back();
        int *has = nullptr, *scan = nullptr;
        if (!dalloc((void**)&has, (size_t)(cnt + 1) * sizeof(int), true) || !dalloc((void**)&scan, (size_t)(cnt + 1) * sizeof(int), true)) {
            release(true);
            return fail("out of device memory", -2);
        }
        cudaMemsetAsync(has, 0, (size_t)(cnt + 1) * sizeof(int), stream);
        k_mark<<<blocks(n, 256), 256, 0, stream>>>(o->scal, n, l, nid, off, has);
        cudaMemcpyAsync(scan, has, (size_t)cnt * sizeof(int), cudaMemcpyDeviceToDevice, stream);
        const int64_t nref = exclusive_scan(scan, cnt, stream);
        const int64_t cnt_next = 8 * nref;
        const int64_t off_next = off + cnt;
        if (cnt_next == 0) break;
        if (off_next + cnt_next >= (1ll << 31) - 16) { release(true); return fail("octree too large for 32-bit node ids", -1); }
        int2* next = nullptr;
        if (!dalloc((void**)&next, (size_t)cnt_next * sizeof(int2), true)) { release(true); return fail("out of device memory", -2); }
        k_children<<<blocks(cnt, 256), 256, 0, stream>>>(cnt, 0, off_next, has, scan, chunks.back(), next);
        k_descend<<<blocks(n, 256), 256, 0, stream>>>(o->keys, o->scal, n, l, nid, nid2, chunks.back(), off, next, off_next,
                                                      cell_node);
        std::swap(nid, nid2);
        chunks.push_back(next);
        counts.push_back(cnt_next);
        offsets.push_back(off_next);
        total = off_next + cnt_next;
    }
    if (!dalloc((void**)&o->node, (size_t)total * sizeof(int2), false)) { release(true); return fail("out of device memory", -2); }
    for (size_t c = 0; c < chunks.size(); ++c)
        cudaMemcpyAsync(o->node + offsets[c], chunks[c], (size_t)counts[c] * sizeof(int2), cudaMemcpyDeviceToDevice, stream);
    o->nnodes = total;
    o->tree.keys = o->keys;
    o->tree.grad = o->grad;
    o->tree.scal = o->scal;
    o->tree.node = o->node;
    o->tree.grid = o->grid;
    o->tree.n = n;
    o->tree.Lt = Lt;
    o->tree.gx0 = bb[0]; o->tree.gy0 = bb[1]; o->tree.gz0 = bb[2];
    o->tree.gnx = gnx; o->tree.gny = gny; o->tree.gnz = gnz;
    if (!dalloc((void**)&o->stencil, (size_t)n * 8 * sizeof(int4), false)) { release(true); return fail("out of device memory", -2); }
    o->tree.stencil = o->stencil;
    k_stencil<<<blocks(n, 128), 128, 0, stream>>>(o->tree, cell_node, o->stencil);
    ce = cudaStreamSynchronize(stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    release(false);
    if (ce != cudaSuccess) { release(true); return fail(cudaGetErrorString(ce), -3); }
    *out = o;
    return 0;
}
