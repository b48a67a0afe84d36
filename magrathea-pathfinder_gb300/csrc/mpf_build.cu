// Cone octree construction from simulation cells, the ASCII path of
// create_octree (Create_octree::PreparationASCII, create_octree.h:544-580),
// on the device:
//
//   Input::importascii (input.h:996-1067)   k_prepare: file level + log2 EXTENT,
//       narrow-cone rotation, the cell key (Index::compute in float, as the
//       reference instantiates it), the cone / sphere filter
//       (Input::collide, input.h:216-226; Utility::collide, utility.h:392-421);
//       order-keeping compaction of the selected cells
//   Input::sistemize (input.h:368-379)      k_sistemize: RAMSES -> SI
//   SimpleHyperOctree::update               radix sort of the 128-bit keys,
//       (simplehyperoctree.h:1270-1310)     k_collapse: cells with one key keep
//                                           the smallest a; dphidt = dphi/da
//   Input::correct (input.h:1381-1516)      coarse densities from their
//       neighbours, refined dphidt / rho from the parent level by level,
//       incomplete octs completed from the gather at the children's centres
//       (k_complete_wave: children filled in waves, each reading only
//       records final before it, so the sequential appends' values result)
//       or, with correction = 0, the coarsening of the parents of refined
//       cells with a non-normal density and of the incomplete octs;
//       acorrection: the scale factors snapped to the next lower one of
//       their table, extended one shell below by a forward derivative
//   correctOctree (miscellaneous.h:467-479) dphidt *= da/dt(a)
//
// Float32 data arithmetic follows the reference's types (Gravity<float, 3>,
// Real = float in importascii); the unit is compiled with -fmad=false and
// its host code without FMA contraction.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpf_gb300.h"
#include "mpf_internal.h"

namespace mpf {
namespace build {

// one cell: the 48-byte cone record (key, Gravity<float, 3>, pad)
struct Rec48 {
    unsigned long long lo, hi;
    float dt, a, dx, dy, dz, phi, rho;
    int pad;
};
static_assert(sizeof(Rec48) == 48, "cone record");

struct Geometry {
    double vertex[3], base[3], angle;
    double sc[3], sr;
    double rot[9];
    int rotate;
    double h, lbox, mpc;
};

__device__ __forceinline__ Key rkey(const Rec48& r) { return Key{r.hi, r.lo}; }

__device__ __forceinline__ bool normal_f(float x)
{
    const float a = fabsf(x);
    return a >= 1.17549435e-38f && a <= 3.40282347e38f;
}

// Index::compute<float, ratio<0>, ratio<EXTENT>> along one axis
__device__ __forceinline__ uint64_t axis_coord_f(int level, float x)
{
    const float scale = (1.0f / 4.0f) * (float)(1ull << level);
    const float v = scale * (x - (-2.0f));
    uint64_t c = (v > 0.0f) ? (uint64_t)v : 0ull;
    return (level >= 64) ? c : (c & ((1ull << level) - 1ull));
}

__device__ __forceinline__ bool collide(const Geometry& G, int L, const double* pos)
{
    // the cell as a sphere of radius extent sqrt(3) / 2
    const double r = cell_extent(L) * sqrt(3.0) / 2.0;
    {
        const double d0 = pos[0] - G.sc[0], d1 = pos[1] - G.sc[1], d2 = pos[2] - G.sc[2];
        if (sqrt(d0 * d0 + (d1 * d1 + (d2 * d2 + 0.0))) < (r + G.sr)) return true;
    }
    double norm = 0.0;
    for (int d = 0; d < 3; ++d) norm += (G.base[d] - G.vertex[d]) * (G.base[d] - G.vertex[d]);
    norm = sqrt(norm);
    double length = 0.0;
    for (int d = 0; d < 3; ++d) length += (G.base[d] - G.vertex[d]) * (pos[d] - G.vertex[d]);
    length /= norm;
    double distance = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = pos[d] - (G.vertex[d] + (G.base[d] - G.vertex[d]) * (length / norm));
        distance += e * e;
    }
    const double R = G.sr;
    const double q = length - R * cos(G.angle);
    return (sqrt(distance) < 5 * r + length * tan(G.angle) + 0.4 * R * exp(-0.7 * q * q / (R * R))) && !(length < 0.0) &&
           (length < norm + r * 2.0);
}

// rows: level x y z rho phi fx fy fz a (floats, as the reference reads them)
__global__ void k_prepare(const float* __restrict__ rows, long long n, Geometry G, int* flag, Rec48* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* w = rows + 10 * i;
    const int L = (int)(unsigned)w[0] + kLevelShift;
    float c[3] = {w[1], w[2], w[3]}, f[3] = {w[6], w[7], w[8]};
    if (G.rotate) {
        const float ct[3] = {c[0], c[1], c[2]}, ft[3] = {f[0], f[1], f[2]};
        for (int r = 0; r < 3; ++r) {
            c[r] = (float)((double)ct[0] * G.rot[3 * r] + (double)ct[1] * G.rot[3 * r + 1] + (double)ct[2] * G.rot[3 * r + 2]);
            f[r] = (float)((double)ft[0] * G.rot[3 * r] + (double)ft[1] * G.rot[3 * r + 1] + (double)ft[2] * G.rot[3 * r + 2]);
        }
    }
    const uint64_t ix = axis_coord_f(L, c[0]), iy = axis_coord_f(L, c[1]), iz = axis_coord_f(L, c[2]);
    const Key k = key_from_coords(L, ix, iy, iz);
    const double pos[3] = {coord_center(L, ix), coord_center(L, iy), coord_center(L, iz)};
    flag[i] = collide(G, L, pos) ? 1 : 0;
    Rec48 r;
    r.lo = k.lo; r.hi = k.hi;
    r.dt = 0.f; r.a = w[9]; r.dx = f[0]; r.dy = f[1]; r.dz = f[2]; r.phi = w[5]; r.rho = w[4];
    r.pad = L;
    out[i] = r;
}

// order-keeping compaction: scan = exclusive prefix sum of flag over n + 1 entries
__global__ void k_select(long long n, const Rec48* __restrict__ in, const int* __restrict__ scan, Rec48* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (scan[i + 1] > scan[i]) out[scan[i]] = in[i];
}

__global__ void k_level_flag(long long n, const Rec48* __restrict__ in, int level, int* flag)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (in[i].pad == level) ? 1 : 0;
}

// Input::sistemize, then dphidt = 0
__global__ void k_sistemize(long long n, Rec48* r, Geometry G)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = (double)r[i].a;
    const double t = (a * a * G.mpc) / (G.h * 100 * 1000);
    const double l = (a * G.lbox * G.mpc) / G.h;
    r[i].phi = (float)((double)r[i].phi * ((l * l) / (t * t)));
    const double g = (l / (t * t)) * (-a);
    r[i].dx = (float)((double)r[i].dx * g);
    r[i].dy = (float)((double)r[i].dy * g);
    r[i].dz = (float)((double)r[i].dz * g);
    r[i].dt = 0.f;
}

// ---- stable LSD radix sort of (hi, lo) with the record index as payload ----
constexpr int kTile = 256;
__global__ void k_keys(long long n, const Rec48* __restrict__ r, unsigned long long* hi, unsigned long long* lo, int* idx)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hi[i] = r[i].hi;
    lo[i] = r[i].lo;
    idx[i] = (int)i;
}
__device__ __forceinline__ unsigned digit(const unsigned long long* hi, const unsigned long long* lo, long long i, int pass)
{
    // passes 0-15 take lo's nibbles from the lowest, 16-31 hi's
    const unsigned long long w = (pass < 16) ? lo[i] : hi[i];
    return (unsigned)((w >> (4 * (pass & 15))) & 15ull);
}
__global__ void k_hist(long long n, const unsigned long long* __restrict__ hi, const unsigned long long* __restrict__ lo,
                       int pass, int* hist, long long ntiles)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    int h[16];
    for (int d = 0; d < 16; ++d) h[d] = 0;
    const long long e = min(n, (t + 1) * kTile);
    for (long long i = t * kTile; i < e; ++i) ++h[digit(hi, lo, i, pass)];
    for (int d = 0; d < 16; ++d) hist[d * ntiles + t] = h[d];
}
__global__ void k_scatter(long long n, const unsigned long long* __restrict__ hi, const unsigned long long* __restrict__ lo,
                          const int* __restrict__ idx, int pass, const int* __restrict__ off, long long ntiles,
                          unsigned long long* hi2, unsigned long long* lo2, int* idx2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    int o[16];
    for (int d = 0; d < 16; ++d) o[d] = off[d * ntiles + t];
    const long long e = min(n, (t + 1) * kTile);
    for (long long i = t * kTile; i < e; ++i) {
        const int j = o[digit(hi, lo, i, pass)]++;
        hi2[j] = hi[i];
        lo2[j] = lo[i];
        idx2[j] = idx[i];
    }
}
__global__ void k_gather(long long n, const Rec48* __restrict__ in, const int* __restrict__ idx, Rec48* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[idx[i]];
}

// SimpleHyperOctree::update's collapse: a run of cells with one key keeps the
// data of its smallest a (the first of them in sorted order) and, when the
// run's a values differ by more than 1e-6, dphidt = (phi - phi') / (a - a')
// between the smallest and the largest a.  flag: 1 on the first of each key.
__global__ void k_collapse(long long n, Rec48* r, int* flag)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Key k = rkey(r[i]);
    const bool head = (i == 0) || !key_eq(rkey(r[i - 1]), k);
    flag[i] = head ? 1 : 0;
    if (!head) return;
    long long e = i + 1;
    while (e < n && key_eq(rkey(r[e]), k)) ++e;
    if (e == i + 1) return;
    long long lo_i = i, hi_i = i;
    for (long long j = i + 1; j < e; ++j) {
        if (r[j].a < r[lo_i].a) lo_i = j;
        if (!(r[j].a < r[hi_i].a)) hi_i = j;
    }
    Rec48 keep = r[lo_i];
    const float fa = r[lo_i].a, ba = r[hi_i].a;
    if (fabs((double)(fa - ba)) > 1e-6) keep.dt = (r[lo_i].phi - r[hi_i].phi) / (fa - ba);
    keep.pad = r[i].pad;
    r[i] = keep;
}

__device__ __forceinline__ void key_coords(Key k, int L, uint64_t* c);

// SimpleHyperOctree::find (simplehyperoctree.h:842-847): the last record with
// a key <= K if it contains K (K itself or an ancestor of K), else -1
__device__ __forceinline__ long long find_containing(const Rec48* r, long long n, Key k, int Lk)
{
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (!key_less(k, rkey(r[mid]))) lo = mid + 1;
        else hi = mid;
    }
    const long long j = lo - (lo > 0);
    if (n <= 0) return -1;
    const int Lj = r[j].pad;
    if (Lj > Lk) return -1;
    uint64_t cj[3], ck[3];
    key_coords(rkey(r[j]), Lj, cj);
    key_coords(k, Lk, ck);
    const int s = Lk - Lj;
    return ((ck[0] >> s) == cj[0] && (ck[1] >> s) == cj[1] && (ck[2] >> s) == cj[2] && key_le(rkey(r[j]), k)) ? j : -1;
}

__device__ __forceinline__ void key_coords(Key k, int L, uint64_t* c)
{
    c[0] = c[1] = c[2] = 0;
    for (int i = 1; i <= L; ++i) {
        const uint64_t nib = (i <= 16) ? (k.hi >> (64 - 4 * i)) & 15ull : (k.lo >> (128 - 4 * i)) & 15ull;
        c[0] = (c[0] << 1) | (nib & 1ull);
        c[1] = (c[1] << 1) | ((nib >> 1) & 1ull);
        c[2] = (c[2] << 1) | ((nib >> 2) & 1ull);
    }
}

// Input::mean over the 26 same-level neighbours with a normal density
// (input.h:244-276), for coarse cells with a non-normal density; rho0 is the
// density before any correction
__global__ void k_coarse_rho(long long n, Rec48* r, const float* __restrict__ rho0, int ncoarse)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (r[i].pad != ncoarse || normal_f(rho0[i])) return;
    const int L = ncoarse;
    uint64_t c[3];
    key_coords(rkey(r[i]), L, c);
    const uint64_t mask = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);
    float result = 0.f;
    unsigned count = 0;
    for (int ix = -1; ix <= 1; ++ix)
        for (int iy = -1; iy <= 1; ++iy)
            for (int iz = -1; iz <= 1; ++iz) {
                if (ix == 0 && iy == 0 && iz == 0) continue;
                const Key nk = key_from_coords(L, (c[0] + (uint64_t)(int64_t)ix) & mask, (c[1] + (uint64_t)(int64_t)iy) & mask,
                                               (c[2] + (uint64_t)(int64_t)iz) & mask);
                const long long j = find_containing(r, n, nk, L);
                if (j >= 0 && normal_f(rho0[j])) {
                    result += rho0[j];
                    ++count;
                }
            }
    r[i].rho = result / (float)(count + (count == 0));
}

__global__ void k_copy_rho(long long n, const Rec48* __restrict__ r, float* rho0)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rho0[i] = r[i].rho;
}

// refined cells of level L whose dphidt (which = 0) or rho (which = 1) is not
// normal take their parent's
__global__ void k_from_parent(long long n, Rec48* r, int L, int which)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (r[i].pad != L) return;
    const float v = which ? r[i].rho : r[i].dt;
    if (normal_f(v)) return;
    uint64_t c[3];
    key_coords(rkey(r[i]), L, c);
    const long long p = find_containing(r, n, key_from_coords(L - 1, c[0] >> 1, c[1] >> 1, c[2] >> 1), L - 1);
    if (p < 0) return;   // the reference dereferences end() there; the cell keeps its value
    if (which) r[i].rho = r[p].rho;
    else r[i].dt = r[p].dt;
}

// non-leaf cells (the next cell is a descendant) with a child that
// SimpleHyperOctree::find does not resolve (no record at or above the child's
// key contains it; a missing child that sorts right after its parent is
// resolved to the parent and not completed, as in the reference): flag = 1
__global__ void k_incomplete(long long n, const Rec48* __restrict__ r, int* flag)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = 0;
    if (i + 1 >= n) return;
    const int L = r[i].pad;
    const Key k = rkey(r[i]), nk = rkey(r[i + 1]);
    // containing: nk's first L levels equal k's and nk is deeper
    const int Ln = r[i + 1].pad;
    if (Ln <= L) return;
    uint64_t c[3], cn[3];
    key_coords(k, L, c);
    key_coords(nk, Ln, cn);
    const int s = Ln - L;
    if ((cn[0] >> s) != c[0] || (cn[1] >> s) != c[1] || (cn[2] >> s) != c[2]) return;
    int missing = 0;
    for (int site = 0; site < 8; ++site) {
        const Key ck = key_from_coords(L + 1, 2 * c[0] + (site & 1), 2 * c[1] + ((site >> 1) & 1), 2 * c[2] + ((site >> 2) & 1));
        missing += (find_containing(r, n, ck, L + 1) < 0);
    }
    flag[i] = missing > 0;
}

// correction = 0 (input.h:1417-1428): a refined cell whose rho is not normal
// marks the cell that SimpleHyperOctree::find returns for its parent key (the
// parent, or the nearest ancestor present); a parent that find does not
// resolve is where the reference coarsens one past its last element, and
// nothing is marked here
__global__ void k_mark_parent(long long n, const Rec48* __restrict__ r, int ncoarse, int* mark)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int L = r[i].pad;
    if (L <= ncoarse || normal_f(r[i].rho)) return;
    uint64_t c[3];
    key_coords(rkey(r[i]), L, c);
    const long long p = find_containing(r, n, key_from_coords(L - 1, c[0] >> 1, c[1] >> 1, c[2] >> 1), L - 1);
    if (p >= 0) mark[p] = 1;
}

// SimpleHyperOctree::coarsen (simplehyperoctree.h:1375-1381) of every marked
// cell, then update's removal of the invalidated ones: coarsen invalidates the
// run of cells after the marked one that it contains, which in key order is
// all of its descendants, so a cell is dropped when a strict ancestor of it is
// marked (coarsening the cells of an already invalidated run in index order
// adds nothing).  keep[i] = 1 for the cells that stay.
__global__ void k_coarsen(long long n, const Rec48* __restrict__ r, const int* __restrict__ mark, int ncoarse, int* keep)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int L = r[i].pad;
    uint64_t c[3];
    key_coords(rkey(r[i]), L, c);
    int k = 1;
    for (int La = L - 1; La >= ncoarse && k; --La) {
        const int s = L - La;
        const Key ak = key_from_coords(La, c[0] >> s, c[1] >> s, c[2] >> s);
        const long long j = find_containing(r, n, ak, La);
        if (j >= 0 && r[j].pad == La && mark[j]) k = 0;
    }
    keep[i] = k;
}

// ---- the reference's gather over a key-sorted array with appended cells ----
// Input::correct appends the children of each incomplete oct at the end of
// the container and gathers the next ones on that container, so the searches
// below run the same binary search (std::upper_bound's loop) over the sorted
// cells plus the unsorted tail.
typedef unsigned __int128 u128;
__device__ __forceinline__ u128 k128(const Rec48& r) { return ((u128)r.hi << 64) | r.lo; }
__device__ __forceinline__ u128 markers128() { return ((u128)0x8888888888888888ull << 64) | 0x8888888888888888ull; }
__device__ __forceinline__ u128 invalid128() { return (((u128)1) << 127) - 1; }
__device__ __forceinline__ unsigned level128(u128 k) { return (unsigned)key_level(Key{(uint64_t)(k >> 64), (uint64_t)k}); }
__device__ __forceinline__ bool containing128(u128 a, u128 b)
{
    const u128 x = a ^ b;
    return ((~markers128() & x) <= (markers128() & x)) && (a <= b);
}
__device__ __forceinline__ u128 parent128(u128 k)
{
    const unsigned loc = 132u - level128(k) * 4u;
    const u128 mask = (loc < 128u) ? (~(u128)0) << loc : (u128)0;
    return k & mask;
}
__device__ __forceinline__ u128 child128(u128 k, unsigned site)
{
    const unsigned l = level128(k);
    if (l >= 32u) return k;
    return k | ((u128)((site & 7u) | 8u) << (128u - (l + 1u) * 4u));
}
__device__ __forceinline__ u128 compute128(unsigned level, double x, double y, double z)
{
    if (level == 0) return 0;
    const Key k = key_from_coords((int)level, axis_coord((int)level, x), axis_coord((int)level, y), axis_coord((int)level, z));
    return ((u128)k.hi << 64) | k.lo;
}
__device__ __forceinline__ double center128(u128 k, int d)
{
    const unsigned l = level128(k);
    uint64_t c[3];
    key_coords(Key{(uint64_t)(k >> 64), (uint64_t)k}, (int)l, c);
    return coord_center((int)l, c[d]);
}
__device__ __forceinline__ long long afind(const Rec48* r, long long n, u128 K)
{
    if (n <= 0) return -1;
    long long first = 0, count = n;
    while (count > 0) {
        const long long step = count >> 1, it = first + step;
        if (!(K < k128(r[it]))) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return (first > 0 && containing128(k128(r[first - 1]), K)) ? first - 1 : -1;
}
// Which records a gather may read.  The completion fills the appended
// children in waves: child j's fields are final once done[j] (the wave that
// filled it) is below the current wave.  A gather that reaches a child not yet
// final is blocked and retried in the next wave; the search paths themselves
// read keys only, which are all written before the first wave.  Without a
// table (done == nullptr) every record is final.
struct Ready {
    const int* done;
    long long m;
    int wave;
    bool blocked;
    __device__ __forceinline__ bool ok(long long i)
    {
        if (done && i >= m && done[i - m] >= wave) blocked = true;
        return !blocked;
    }
};
__device__ __forceinline__ void afields(const Rec48& r, float* f)
{
    f[0] = r.rho; f[1] = r.phi; f[2] = r.dx; f[3] = r.dy; f[4] = r.dz; f[5] = r.a; f[6] = r.dt;
}
__device__ __forceinline__ void amac(float* acc, const float* f, double w)
{
    for (int q = 0; q < 7; ++q) acc[q] = (float)((double)acc[q] + (double)f[q] * w);
}
__device__ __forceinline__ void azero(float* a)
{
    for (int q = 0; q < 7; ++q) a[q] = 0.f;
}
// SimpleHyperOctree::ngp (simplehyperoctree.h:1396-1401) over the array: the
// record the containing search finds at the position's level-32 key
__device__ void angp(const Rec48* r, long long n, double x, double y, double z, float* res, Ready& rd)
{
    const long long f0 = afind(r, n, compute128(32, x, y, z));
    if (f0 >= 0 && !rd.ok(f0)) return;
    if (f0 >= 0) afields(r[f0], res);
    else azero(res);
}
// SimpleHyperOctree::cic (simplehyperoctree.h:1410-1469) over the array
__device__ void acic(const Rec48* r, long long n, double x, double y, double z, float* res, Ready& rd)
{
    const double pt[3] = {x, y, z};
    u128 ekey = compute128(32, x, y, z);
    const long long f0 = afind(r, n, ekey);
    u128 idx = (f0 >= 0) ? k128(r[f0]) : invalid128();
    unsigned ilvl = level128(idx), lvl = ilvl;
    double half = 4.0 / 1.0 * (1.0 / (1.0 * (double)(((u128)1) << level128(idx)))) / 2.0;
    unsigned site = 0;
    azero(res);
    for (int guard = 0; guard <= 33; ++guard) {
        ilvl = lvl;
        if (idx != invalid128()) {
            double dist[3];
            for (int d = 0; d < 3; ++d) dist[d] = fabs((center128(idx, d) - pt[d]) / (half + half));
            for (unsigned s2 = 0; s2 < 8u; ++s2)
                if (containing128(child128(idx, s2), ekey)) { site = s2; break; }
            for (unsigned v = 0; v < 8u; ++v) {
                double w = 1.0, vert[3];
                const unsigned diff = site ^ v;
                for (int d = 0; d < 3; ++d) {
                    const int b = (v >> d) & 1u, db = (diff >> d) & 1u;
                    vert[d] = pt[d] + ((double)b * half) - ((double)(!b) * half);
                    w *= ((double)db * (1.0 - dist[d])) + ((double)(!db) * dist[d]);
                }
                ekey = compute128(ilvl, vert[0], vert[1], vert[2]);
                const long long fi = afind(r, n, ekey);
                if (fi >= 0) {
                    if (!rd.ok(fi)) return;
                    const unsigned fl = level128(k128(r[fi]));
                    if (fl < lvl) lvl = fl;
                    float f[7];
                    afields(r[fi], f);
                    amac(res, f, w);
                } else {
                    azero(res);
                    break;
                }
            }
        }
        if (lvl < ilvl) {
            ekey = compute128(lvl + 1, x, y, z);
            idx = parent128(ekey);
            azero(res);
            half = 4.0 / 1.0 * (1.0 / (1.0 * (double)(((u128)1) << level128(idx)))) / 2.0;
        } else {
            break;
        }
    }
}
__device__ __forceinline__ double tsc_weight(int a, double d)
{
    return (double)a * 0.5 * (1.5 - d) * (1.5 - d) + (double)(1 - a) * (0.75 - d * d);
}
// SimpleHyperOctree::tsc (simplehyperoctree.h:1479-1541) over the array
__device__ void atsc(const Rec48* r, long long n, double x, double y, double z, float* res, Ready& rd)
{
    const double pt[3] = {x, y, z};
    u128 ekey = compute128(32, x, y, z);
    const long long f0 = afind(r, n, ekey);
    u128 idx = (f0 >= 0) ? k128(r[f0]) : invalid128();
    unsigned ilvl = level128(idx), lvl = ilvl;
    double half = 4.0 / 1.0 * (1.0 / (1.0 * (double)(((u128)1) << level128(idx)))) / 2.0;
    azero(res);
    if (x == 0.0 && y == 0.0 && z == 0.0) {
        acic(r, n, 0., 0., 0., res, rd);
        return;
    }
    for (int guard = 0; guard <= 33; ++guard) {
        ilvl = lvl;
        const double tw = 2.0 * half;
        if (idx != invalid128()) {
            bool stop = false;
            for (int ix = -1; ix <= 1 && !stop; ++ix)
                for (int iy = -1; iy <= 1 && !stop; ++iy)
                    for (int iz = -1; iz <= 1 && !stop; ++iz) {
                        ekey = compute128(ilvl, pt[0] + ix * tw, pt[1] + iy * tw, pt[2] + iz * tw);
                        const long long fi = afind(r, n, ekey);
                        if (fi >= 0) {
                            if (!rd.ok(fi)) return;
                            float f[7];
                            afields(r[fi], f);
                            double dist[3];
                            for (int d = 0; d < 3; ++d) dist[d] = fabs((center128(ekey, d) - pt[d]) / tw);
                            const double w = tsc_weight(abs(ix), dist[0]) * tsc_weight(abs(iy), dist[1]) * tsc_weight(abs(iz), dist[2]);
                            const unsigned fl = level128(k128(r[fi]));
                            if (fl < lvl) lvl = fl;
                            if (lvl < ilvl) { azero(res); stop = true; }
                            else amac(res, f, w);
                        } else {
                            azero(res);
                            stop = true;
                        }
                    }
        }
        if (lvl < ilvl) {
            ekey = compute128(lvl + 1, x, y, z);
            idx = parent128(ekey);
            azero(res);
            half = 4.0 / 1.0 * (1.0 / (1.0 * (double)(((u128)1) << level128(idx)))) / 2.0;
        } else {
            break;
        }
    }
}

// Input::correct's completion loop (input.h:1451-1482): for each incomplete
// cell (key order) its 8 children are gathered at their centres on the array
// as it stands -- the children appended before included -- and appended.
// Child c (parent c / 8, site c % 8) is therefore gathered over the first
// m + c records.  Which records a search visits depends on keys alone, and
// every appended key is known before any gather, so the children are filled
// in waves: in each wave every child whose gather reads only prefix records
// or children of earlier waves is final; the others retry.  The lowest
// unfilled child always completes (its reads are all earlier children), and
// what a bounded number of waves leaves is filled in order on one thread.
// Every child reads the same records with the same values as in the
// sequential loop, so the result is the same bit for bit.

// the appended children: key, level and the parent's fields (kept when the
// gather is empty), all unfilled
__global__ void k_complete_init(Rec48* r, long long m, const int* __restrict__ list, long long nch, int* done)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nch) return;
    Rec48 o = r[list[c >> 3]];
    const u128 ck = child128(k128(o), (unsigned)(c & 7));
    o.hi = (unsigned long long)(ck >> 64);
    o.lo = (unsigned long long)ck;
    o.pad += 1;
    r[m + c] = o;
    done[c] = INT_MAX;
}

// child c's gather at its centre over the first m + c records; its fields
// (not its key, which other gathers read meanwhile) written when non-empty
__device__ bool complete_child(Rec48* r, long long m, long long c, int order, Ready& rd)
{
    const u128 ck = k128(r[m + c]);
    // the child's centre as the reference computes it, in float
    const float cx = (float)center128(ck, 0), cy = (float)center128(ck, 1), cz = (float)center128(ck, 2);
    float f[7];
    if (order == 0) angp(r, m + c, cx, cy, cz, f, rd);
    else if (order == 1) acic(r, m + c, cx, cy, cz, f, rd);
    else atsc(r, m + c, cx, cy, cz, f, rd);
    if (rd.blocked) return false;
    bool empty = true;
    for (int k = 0; k < 7; ++k) empty = empty && (f[k] == 0.f);
    if (!empty) {
        Rec48& o = r[m + c];
        o.rho = f[0]; o.phi = f[1]; o.dx = f[2]; o.dy = f[3]; o.dz = f[4]; o.a = f[5]; o.dt = f[6];
    }
    return true;
}

__global__ void k_complete_wave(Rec48* r, long long m, long long nch, int order, int* done, int wave, int* pending)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nch || done[c] != INT_MAX) return;
    Ready rd{done, m, wave, false};
    if (complete_child(r, m, c, order, rd)) done[c] = wave;
    else atomicAdd(pending, 1);
}

// what the waves left, in the sequential order
__global__ void k_complete_rest(Rec48* r, long long m, long long nch, int order, const int* __restrict__ done)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (long long c = 0; c < nch; ++c) {
        if (done[c] != INT_MAX) continue;
        Ready rd{nullptr, m, 0, false};
        complete_child(r, m, c, order, rd);
    }
}

// Utility::interpolate2 (utility.h:461-468): descending table, float result
__device__ __forceinline__ float interpolate2(float x0, const double* x, const double* y, long long n)
{
    long long first = 0, count = n;
    while (count > 0) {
        const long long step = count >> 1, it = first + step;
        if (!((double)x0 > x[it])) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    long long i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n > 1) return (float)(y[i - 1] + ((y[i] - y[i - 1]) * ((double)x0 - x[i - 1]) / (x[i] - x[i - 1])));
    return (n > 0) ? (float)y[0] : 0.f;
}

// acorrection (input.h:1485-1506), the Full Universe Run scale-factor
// snapping.  The cells' scale factors as sortable 32-bit keys (non-negative
// floats order as their bit patterns); the values the reference drops from its
// table (sign bit set, or not normal) get 0xffffffff and sort last.
__global__ void k_a_keys(long long n, const Rec48* __restrict__ r, unsigned long long* hi, unsigned long long* lo, int* idx)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = r[i].a;
    hi[i] = 0ull;
    lo[i] = (!signbit(a) && normal_f(a)) ? (unsigned long long)__float_as_uint(a) : 0xffffffffull;
    idx[i] = (int)i;
}

// the first of each run of equal sorted keys, the dropped values excluded
__global__ void k_a_unique(long long n, const unsigned long long* __restrict__ lo, int* flag)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (lo[i] != 0xffffffffull && (i == 0 || lo[i] != lo[i - 1])) ? 1 : 0;
}

__global__ void k_a_select(long long n, const unsigned long long* __restrict__ lo, const int* __restrict__ scan, float* table)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (scan[i + 1] > scan[i]) table[scan[i]] = __uint_as_float((unsigned)lo[i]);
}

// each cell's a becomes the table's value below it, *(lower_bound(a) - 1);
// a cell whose a is the table's first value or was dropped from the table
// reads before the table in the reference (undefined) and keeps its a here
__global__ void k_a_snap(long long n, Rec48* r, const float* __restrict__ table, int T)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = r[i].a;
    int lo = 0, hi = T;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (table[mid] < a) lo = mid + 1;
        else hi = mid;
    }
    if (lo > 0) r[i].a = table[lo - 1];
}

__global__ void k_dphidt(long long n, Rec48* r, const double* __restrict__ ca, const double* __restrict__ cdadt, long long nc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    r[i].dt *= interpolate2(r[i].a, ca, cdadt, nc);
    r[i].pad = 0;
}

inline unsigned blk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace build
}  // namespace mpf

using namespace mpf;
using namespace mpf::build;

namespace {
int fail(int code, const std::string& m) { return mpf_internal_set_error(code, m.c_str()); }

struct Arena {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* get(size_t count)
    {
        void* p = nullptr;
        if (err == cudaSuccess && count) err = cudaMalloc(&p, count * sizeof(T));
        if (p) ptrs.push_back(p);
        return (T*)p;
    }
    ~Arena()
    {
        for (void* p : ptrs) cudaFree(p);
    }
};

// Utility::interpolate (utility.h:440-447) over float tables: upper_bound,
// then the bracketing segment, clamped to the end segments
float interpolate_f(float x0, const std::vector<float>& x, const std::vector<float>& y)
{
    const long long n = (long long)std::min(x.size(), y.size());
    long long i = std::upper_bound(x.begin(), x.begin() + n, x0) - x.begin();
    i += (n > 1) * ((i <= 0) - (i >= n));
    return (n > 1) ? (y[i - 1] + ((y[i] - y[i - 1]) * (x0 - x[i - 1]) / (x[i] - x[i - 1]))) : ((n > 0) ? y[0] : 0.f);
}

// Utility::differentiate<1> (utility.h:527-551) with neighbourhood 1: the
// nine-point one-sided (forward) finite-difference weights of Fornberg's
// method, step = the abscissae's spacing at x0, in float
float forward_derivative_f(float x0, const std::vector<float>& x, const std::vector<float>& y)
{
    const float w[9] = {-761.f / 280.f, 8.f, -14.f, 56.f / 3.f, -35.f / 2.f, 56.f / 5.f, -14.f / 3.f, 8.f / 7.f, -1.f / 8.f};
    const long long n = (long long)std::min(x.size(), y.size());
    const long long i = std::upper_bound(x.begin(), x.begin() + n, x0) - x.begin();
    const long long j = i + ((n > 1) * ((i <= 0) - (i >= n)));
    const float h = (n > 1) ? ((x[j] - x[j - 1]) * 1u) : 0.f;
    float result = 0.f;
    if (n > 1)
        for (int k = 0; k < 9; ++k) result += w[8 - k] * interpolate_f(x0 + (float)(8 - k) * h, x, y);
    return result / h;
}

// compact `in` (n records) by flag into out; returns the count
long long compact(Arena& A, const Rec48* in, long long n, int* flag, Rec48* out, cudaStream_t s)
{
    cudaMemsetAsync(flag + n, 0, sizeof(int), s);
    const long long total = exclusive_scan(flag, n + 1, s);
    k_select<<<blk(n, 256), 256, 0, s>>>(n, in, flag, out);
    return total;
}

// sort n records by key (stable) into out
void sort_records(Arena& A, const Rec48* in, long long n, Rec48* out, cudaStream_t s)
{
    unsigned long long *hi = A.get<unsigned long long>(n), *lo = A.get<unsigned long long>(n);
    unsigned long long *hi2 = A.get<unsigned long long>(n), *lo2 = A.get<unsigned long long>(n);
    int *idx = A.get<int>(n), *idx2 = A.get<int>(n);
    const long long ntiles = (n + kTile - 1) / kTile;
    int* hist = A.get<int>((size_t)16 * ntiles + 1);
    if (A.err != cudaSuccess) return;
    k_keys<<<blk(n, 256), 256, 0, s>>>(n, in, hi, lo, idx);
    for (int pass = 0; pass < 32; ++pass) {
        k_hist<<<blk(ntiles, 128), 128, 0, s>>>(n, hi, lo, pass, hist, ntiles);
        exclusive_scan(hist, 16 * ntiles, s);
        k_scatter<<<blk(ntiles, 128), 128, 0, s>>>(n, hi, lo, idx, pass, hist, ntiles, hi2, lo2, idx2);
        std::swap(hi, hi2);
        std::swap(lo, lo2);
        std::swap(idx, idx2);
    }
    k_gather<<<blk(n, 256), 256, 0, s>>>(n, in, idx, out);
}

// Input::correct's acorrection over the n records of r as the container
// holds them then (appended or invalidated cells included): the table of
// the distinct scale factors (sorted on the device), one shell below it
// extrapolated against the table's index (1, 2, ...) when that gives a
// positive normal value below the first, then every cell's a snapped to the
// table value below it.  amin: the table's first value.
cudaError_t acorrect(Arena& A, Rec48* r, long long n, double* amin, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    // the table of the cells' distinct scale factors, sorted on the device
    unsigned long long *hi = A.get<unsigned long long>(n), *lo = A.get<unsigned long long>(n);
    unsigned long long *hi2 = A.get<unsigned long long>(n), *lo2 = A.get<unsigned long long>(n);
    int *idx = A.get<int>(n), *idx2 = A.get<int>(n), *uflag = A.get<int>(n + 1);
    float* dtable = A.get<float>(n + 1);
    const long long ntiles = (n + kTile - 1) / kTile;
    int* hist = A.get<int>((size_t)16 * ntiles + 1);
    if (A.err != cudaSuccess) return A.err;
    k_a_keys<<<blk(n, 256), 256, 0, s>>>(n, r, hi, lo, idx);
    for (int pass = 0; pass < 8; ++pass) {
        k_hist<<<blk(ntiles, 128), 128, 0, s>>>(n, hi, lo, pass, hist, ntiles);
        exclusive_scan(hist, 16 * ntiles, s);
        k_scatter<<<blk(ntiles, 128), 128, 0, s>>>(n, hi, lo, idx, pass, hist, ntiles, hi2, lo2, idx2);
        std::swap(hi, hi2);
        std::swap(lo, lo2);
        std::swap(idx, idx2);
    }
    k_a_unique<<<blk(n, 256), 256, 0, s>>>(n, lo, uflag);
    cudaMemsetAsync(uflag + n, 0, sizeof(int), s);
    const long long asize = exclusive_scan(uflag, n + 1, s);
    k_a_select<<<blk(n, 256), 256, 0, s>>>(n, lo, uflag, dtable);
    std::vector<float> table((size_t)asize);
    cudaError_t e = cudaSuccess;
    if (asize > 0) e = cudaMemcpy(table.data(), dtable, (size_t)asize * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    // one shell below the first, extrapolated from the table against its
    // index (1, 2, ...) when that gives a positive normal value below it
    if (asize > 1) {
        std::vector<float> index((size_t)asize);
        for (long long k = 0; k < asize; ++k) index[(size_t)k] = (float)(k + 1);
        const float below = table[0] - forward_derivative_f(0.f, index, table);
        if (!std::signbit(below) && std::isnormal(below) && below < table[0]) table.insert(table.begin(), below);
    }
    if (!table.empty()) {
        e = cudaMemcpy(dtable, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        k_a_snap<<<blk(n, 256), 256, 0, s>>>(n, r, dtable, (int)table.size());
        if (amin) *amin = (double)table[0];
    }
    return cudaGetLastError();
}

// SimpleHyperOctree::update on device records: sort, collapse, compact
long long update(Arena& A, Rec48* r, long long n, Rec48* tmp, int* flag, cudaStream_t s)
{
    sort_records(A, r, n, tmp, s);
    if (A.err != cudaSuccess) return -1;
    k_collapse<<<blk(n, 256), 256, 0, s>>>(n, tmp, flag);
    return compact(A, tmp, n, flag, r, s);
}
}  // namespace

// the completion of the calling thread's last mpf_cells_build: incomplete
// cells, children filled in waves, waves run, children filled in order after
// them
namespace {
struct Completion {
    long long incomplete, in_waves;
    int waves;
    long long sequential;
};
thread_local Completion g_completion = {0, 0, 0, 0};

// MPF_COMPLETION_WAVES: the most waves before the sequential fill (default
// 32; 0 fills every child in order on one thread)
int completion_waves()
{
    const char* v = std::getenv("MPF_COMPLETION_WAVES");
    if (!v || !*v) return 32;
    return std::min(std::max(std::atoi(v), 0), 4096);
}
}  // namespace

extern "C" int mpf_cells_completion_info(int64_t* info)
{
    if (!info) return fail(MPF_BAD_INPUT, "mpf_cells_completion_info: bad argument");
    info[0] = g_completion.incomplete;
    info[1] = g_completion.in_waves;
    info[2] = g_completion.waves;
    info[3] = g_completion.sequential;
    return MPF_OK;
}

extern "C" int mpf_cells_build(const float* rows, int64_t n, const mpf_cells_params* cp, const mpf_cosmology* c, void* records,
                               int64_t capacity, int64_t* count)
{
    g_completion = {0, 0, 0, 0};
    const int max_waves = completion_waves();
    if ((n > 0 && !rows) || n < 0 || !cp || !c || !count || (capacity > 0 && !records))
        return fail(MPF_BAD_INPUT, "mpf_cells_build: bad argument");
    if (cp->order < 0 || cp->order > 2) return fail(MPF_BAD_INPUT, "mpf_cells_build: order must be 0, 1 or 2");
    if (n == 0) {   // no cell files for this cone: an empty octree, as the reference saves it
        *count = 0;
        return MPF_OK;
    }
    Geometry G;
    std::memset(&G, 0, sizeof(G));
    for (int d = 0; d < 3; ++d) {
        G.vertex[d] = cp->cone_vertex[d];
        G.base[d] = cp->cone_base[d];
        G.sc[d] = cp->sphere_center[d];
    }
    G.angle = cp->cone_angle;
    G.sr = cp->sphere_radius;
    G.rotate = cp->rotm1 != nullptr;
    if (cp->rotm1)
        for (int q = 0; q < 9; ++q) G.rot[q] = cp->rotm1[q];
    G.h = cp->h;
    G.lbox = cp->lboxmpch;
    G.mpc = cp->mpc;
    cudaStream_t s = 0;
    Arena A;
    float* drows = A.get<float>((size_t)n * 10);
    Rec48 *r0 = A.get<Rec48>(n), *r1 = A.get<Rec48>(n);
    int* flag = A.get<int>(n + 1);
    if (A.err != cudaSuccess) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
    cudaError_t e = cudaMemcpy(drows, rows, (size_t)n * 10 * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
    // importascii: keys, filter, compaction (file order kept)
    k_prepare<<<blk(n, 256), 256, 0, s>>>(drows, n, G, flag, r0);
    long long m = compact(A, r0, n, flag, r1, s);
    if (cp->coarseonly) {
        k_level_flag<<<blk(m, 256), 256, 0, s>>>(m, r1, cp->ncoarse + kLevelShift, flag);
        m = compact(A, r1, m, flag, r0, s);
        std::swap(r0, r1);
    }
    if (m <= 0) {
        *count = 0;
        return MPF_OK;
    }
    // sistemize, dphidt = 0, update
    k_sistemize<<<blk(m, 256), 256, 0, s>>>(m, r1, G);
    m = update(A, r1, m, r0, flag, s);
    if (A.err != cudaSuccess || m < 0) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
    // Input::correct
    std::vector<Rec48> h((size_t)m);
    e = cudaMemcpy(h.data(), r1, (size_t)m * sizeof(Rec48), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
    int ncoarse = 64, nmax = 0;
    for (const Rec48& x : h) {
        ncoarse = std::min(ncoarse, x.pad);
        nmax = std::max(nmax, x.pad);
    }
    if (cp->coarsecorrection) {
        float* rho0 = A.get<float>(m);
        if (A.err != cudaSuccess) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
        k_copy_rho<<<blk(m, 256), 256, 0, s>>>(m, r1, rho0);
        k_coarse_rho<<<blk(m, 128), 128, 0, s>>>(m, r1, rho0, ncoarse);
    }
    if (!cp->correction) {
        // refined cells with a non-normal rho: their parents coarsened, then
        // the incomplete octs coarsened too (input.h:1417-1428, 1472-1481)
        int* mark = A.get<int>(m);
        if (A.err != cudaSuccess) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
        cudaMemsetAsync(mark, 0, (size_t)m * sizeof(int), s);
        k_mark_parent<<<blk(m, 256), 256, 0, s>>>(m, r1, ncoarse, mark);
        k_coarsen<<<blk(m, 128), 128, 0, s>>>(m, r1, mark, ncoarse, flag);
        m = compact(A, r1, m, flag, r0, s);
        k_incomplete<<<blk(m, 128), 128, 0, s>>>(m, r0, mark);
        k_coarsen<<<blk(m, 128), 128, 0, s>>>(m, r0, mark, ncoarse, flag);
        // the invalidated cells stay in the container until the final update
        if (cp->acorrection && (e = acorrect(A, r0, m, cp->amin, s)) != cudaSuccess)
            return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
        m = compact(A, r0, m, flag, r1, s);
    } else {
        for (int L = ncoarse + 1; L <= nmax; ++L) k_from_parent<<<blk(m, 256), 256, 0, s>>>(m, r1, L, 0);
        for (int L = ncoarse + 1; L <= nmax; ++L) k_from_parent<<<blk(m, 256), 256, 0, s>>>(m, r1, L, 1);
    }
    // incomplete octs: the 8 children from the gather on the octree so far
    long long ninc = 0;
    if (cp->correction) {
        k_incomplete<<<blk(m, 128), 128, 0, s>>>(m, r1, flag);
        cudaMemsetAsync(flag + m, 0, sizeof(int), s);
        ninc = exclusive_scan(flag, m + 1, s);
    }
    if (ninc > 0) {
        int* list = A.get<int>(ninc);
        Rec48* grown = A.get<Rec48>(m + 8 * ninc);
        Rec48* tmp = A.get<Rec48>(m + 8 * ninc);
        int* flag2 = A.get<int>(m + 8 * ninc + 1);
        if (A.err != cudaSuccess) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
        // the list of incomplete cells, in key order
        std::vector<int> hflag((size_t)m + 1), hl;
        cudaMemcpy(hflag.data(), flag, (size_t)(m + 1) * sizeof(int), cudaMemcpyDeviceToHost);
        for (long long i = 0; i < m; ++i)
            if (hflag[i + 1] > hflag[i]) hl.push_back((int)i);
        cudaMemcpy(list, hl.data(), hl.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(grown, r1, (size_t)m * sizeof(Rec48), cudaMemcpyDeviceToDevice);
        const long long nch = 8 * ninc;
        int* done = A.get<int>(nch);
        int* pending = A.get<int>(std::max(max_waves, 1));
        if (A.err != cudaSuccess) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
        cudaMemsetAsync(pending, 0, (size_t)std::max(max_waves, 1) * sizeof(int), s);
        k_complete_init<<<blk(nch, 128), 128, 0, s>>>(grown, m, list, nch, done);
        long long left = nch;
        int wave = 0;
        while (left > 0 && wave < max_waves) {
            ++wave;
            k_complete_wave<<<blk(nch, 128), 128, 0, s>>>(grown, m, nch, cp->order, done, wave, pending + wave - 1);
            int h_left = 0;
            e = cudaMemcpyAsync(&h_left, pending + wave - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
            left = h_left;
        }
        if (left > 0) k_complete_rest<<<1, 1, 0, s>>>(grown, m, nch, cp->order, done);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
        g_completion = {ninc, nch - left, wave, left};
        // acorrection runs on the container with its appended children, before the final update
        if (cp->acorrection && (e = acorrect(A, grown, m + 8 * ninc, cp->amin, s)) != cudaSuccess)
            return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
        m = update(A, grown, m + 8 * ninc, tmp, flag2, s);
        if (A.err != cudaSuccess || m < 0) return fail(MPF_OUT_OF_MEMORY, "mpf_cells_build: device memory");
        r1 = grown;
    } else if (cp->correction && cp->acorrection && (e = acorrect(A, r1, m, cp->amin, s)) != cudaSuccess) {
        return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
    }
    // dphidt *= da/dt at the cell's a
    k_dphidt<<<blk(m, 256), 256, 0, s>>>(m, r1, c->a, c->dadt, c->n);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
    *count = m;
    if (m > capacity) return fail(MPF_BAD_INPUT, "mpf_cells_build: more cells than capacity (see count)");
    e = cudaMemcpy(records, r1, (size_t)m * sizeof(Rec48), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(MPF_CUDA_ERROR, std::string("mpf_cells_build: ") + cudaGetErrorString(e));
    return MPF_OK;
}

extern "C" int mpf_cells_parse(const char* text, int64_t length, float* rows, int64_t capacity, int64_t* count)
{
    if (!text || length < 0 || !count || (capacity > 0 && !rows)) return fail(MPF_BAD_INPUT, "mpf_cells_parse: bad argument");
    // whitespace-separated: an unsigned level then 9 floats per cell (the
    // reference's stream >> unsigned >> float ... reads)
    std::string buf(text, (size_t)length);
    const char* p = buf.c_str();
    char* end = nullptr;
    int64_t k = 0;
    for (;;) {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
        if (!*p) break;
        float v[10];
        const unsigned long lv = std::strtoul(p, &end, 10);
        if (end == p) return fail(MPF_BAD_INPUT, "mpf_cells_parse: malformed level");
        p = end;
        v[0] = (float)lv;
        for (int q = 1; q < 10; ++q) {
            v[q] = std::strtof(p, &end);
            if (end == p) return fail(MPF_BAD_INPUT, "mpf_cells_parse: malformed row");
            p = end;
        }
        if (k < capacity)
            for (int q = 0; q < 10; ++q) rows[10 * k + q] = v[q];
        ++k;
    }
    *count = k;
    return (k > capacity) ? fail(MPF_BAD_INPUT, "mpf_cells_parse: more rows than capacity (see count)") : MPF_OK;
}
