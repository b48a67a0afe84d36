/* CPU oracle, octree build: plain-C restatement of the reference's cone
 * octree construction from ASCII cells (Create_octree::PreparationASCII's
 * per-cone body).  TEST INFRASTRUCTURE ONLY (see mpf_oracle.h).  Build with
 * -ffp-contract=off.
 *
 * Sources restated (reference paths):
 *   rows              src/input.h:996-1067 (Input::importascii: file level
 *                     + log2 EXTENT, narrow-cone rotation, the key of the
 *                     float position, Input::collide)
 *   cone filter       src/input.h:216-226, src/utility.h:392-421
 *   sistemize         src/input.h:368-379
 *   update            src/magrathea/simplehyperoctree.h:1270-1310 (stable
 *                     sort by key, the run of one key keeps its smallest a,
 *                     dphidt = dphi / da between the smallest and largest a)
 *   find              src/magrathea/simplehyperoctree.h:842-847
 *   correct           src/input.h:1381-1516 (coarse densities from the
 *                     neighbours' mean, :244-276; refined dphidt / rho from
 *                     the parent; the completion of incomplete octs by the
 *                     gathers of cic / tsc / ngp at the children's centres
 *                     over the growing container; with correction = 0 the
 *                     coarsening of the parents of refined cells with a
 *                     non-normal density and of the incomplete octs,
 *                     simplehyperoctree.h:1375-1381; acorrection)
 *   gathers           src/magrathea/simplehyperoctree.h:1396-1401 (ngp),
 *                     :1410-1469 (cic), :1479-1541 (tsc, uncached)
 *   interpolate       src/utility.h:440-447 (float), :461-468 (interpolate2)
 *   differentiate     src/utility.h:527-551 (forward, neighbourhood 1)
 *   correctOctree     src/miscellaneous.h:467-479 (dphidt *= da/dt(a))
 */
#include "mpf_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mpf_oracle_keys.h"

/* the 48-byte cone record: key (lo, hi), Gravity<float, 3>'s fields, pad
 * (the cell's level while the octree is built) */
typedef struct {
    uint64_t lo, hi;
    float dt, a, dx, dy, dz, phi, rho;
    int32_t pad;
} rec48;
_Static_assert(sizeof(rec48) == 48, "cone record");

static inline u128 rkey(const rec48* r) { return mk(r->hi, r->lo); }

static inline int normal_f(float x)
{
    const float a = fabsf(x);
    return a >= FLT_MIN && a <= FLT_MAX;
}

/* Index::compute<float, ratio<0>, ratio<EXTENT>> along one axis */
static inline uint64_t axis_coord_f(int level, float x)
{
    const float scale = (1.0f / 4.0f) * (float)(1ULL << level);
    const float v = scale * (x - (-2.0f));
    const uint64_t c = (v > 0.0f) ? (uint64_t)v : 0ULL;
    return (level >= 64) ? c : (c & ((1ULL << level) - 1ULL));
}

static u128 key_of_coords(int L, uint64_t cx, uint64_t cy, uint64_t cz)
{
    u128 k = 0;
    for (int i = 1; i <= L; ++i) {
        const int b = L - i;
        const unsigned nib = 8u | (unsigned)(((cz >> b) & 1u) << 2) | (unsigned)(((cy >> b) & 1u) << 1) |
                             (unsigned)((cx >> b) & 1u);
        k |= (u128)nib << (128 - 4 * i);
    }
    return k;
}

static void coords_of_key(u128 k, int L, uint64_t* c)
{
    c[0] = c[1] = c[2] = 0;
    for (int i = 1; i <= L; ++i) {
        const unsigned nib = (unsigned)(k >> (128 - 4 * i)) & 15u;
        c[0] = (c[0] << 1) | (nib & 1u);
        c[1] = (c[1] << 1) | ((nib >> 1) & 1u);
        c[2] = (c[2] << 1) | ((nib >> 2) & 1u);
    }
}

/* Utility::collide of the cell (a sphere of radius extent * sqrt(3) / 2)
 * with the microsphere and the cone */
static int collide(const mpfo_cells_params* P, int L, const double* pos)
{
    const double r = ((double)OCT_EXTENT / (1.0 * (double)(((u128)1) << L))) * sqrt(3.0) / 2.0;
    {
        const double d0 = pos[0] - P->sphere_center[0], d1 = pos[1] - P->sphere_center[1], d2 = pos[2] - P->sphere_center[2];
        if (sqrt(d0 * d0 + (d1 * d1 + (d2 * d2 + 0.0))) < (r + P->sphere_radius)) return 1;
    }
    double norm = 0.0;
    for (int d = 0; d < 3; ++d) norm += (P->cone_base[d] - P->cone_vertex[d]) * (P->cone_base[d] - P->cone_vertex[d]);
    norm = sqrt(norm);
    double length = 0.0;
    for (int d = 0; d < 3; ++d) length += (P->cone_base[d] - P->cone_vertex[d]) * (pos[d] - P->cone_vertex[d]);
    length /= norm;
    double distance = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = pos[d] - (P->cone_vertex[d] + (P->cone_base[d] - P->cone_vertex[d]) * (length / norm));
        distance += e * e;
    }
    const double R = P->sphere_radius;
    const double q = length - R * cos(P->cone_angle);
    return (sqrt(distance) < 5 * r + length * tan(P->cone_angle) + 0.4 * R * exp(-0.7 * q * q / (R * R))) &&
           !(length < 0.0) && (length < norm + r * 2.0);
}

/* SimpleHyperOctree::find over sorted records: the last record with a key
 * <= K if it contains K (K itself or an ancestor), else -1 */
static int64_t find_containing(const rec48* r, int64_t n, u128 K, int LK)
{
    if (n <= 0) return -1;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (!(K < rkey(&r[mid]))) lo = mid + 1;
        else hi = mid;
    }
    const int64_t j = lo - (lo > 0);
    const int Lj = r[j].pad;
    if (Lj > LK) return -1;
    uint64_t cj[3], ck[3];
    coords_of_key(rkey(&r[j]), Lj, cj);
    coords_of_key(K, LK, ck);
    const int s = LK - Lj;
    return ((ck[0] >> s) == cj[0] && (ck[1] >> s) == cj[1] && (ck[2] >> s) == cj[2] && rkey(&r[j]) <= K) ? j : -1;
}

/* ---- SimpleHyperOctree::update: stable sort, collapse, compaction ---- */
typedef struct {
    u128 k;
    int64_t i;
} sort_item;

static int by_key_then_index(const void* a, const void* b)
{
    const sort_item *x = (const sort_item*)a, *y = (const sort_item*)b;
    if (x->k != y->k) return (x->k < y->k) ? -1 : 1;
    return (x->i < y->i) ? -1 : (x->i > y->i);
}

/* sorts r[0, n) by key (stable) and collapses each run of one key; returns
 * the new count, or -1 without memory */
static int64_t update(rec48* r, int64_t n)
{
    if (n <= 0) return 0;
    sort_item* it = (sort_item*)malloc((size_t)n * sizeof(sort_item));
    rec48* s = (rec48*)malloc((size_t)n * sizeof(rec48));
    if (!it || !s) {
        free(it);
        free(s);
        return -1;
    }
    for (int64_t i = 0; i < n; ++i) {
        it[i].k = rkey(&r[i]);
        it[i].i = i;
    }
    qsort(it, (size_t)n, sizeof(sort_item), by_key_then_index);
    for (int64_t i = 0; i < n; ++i) s[i] = r[it[i].i];
    int64_t m = 0;
    for (int64_t i = 0; i < n;) {
        int64_t e = i + 1;
        while (e < n && rkey(&s[e]) == rkey(&s[i])) ++e;
        rec48 keep = s[i];
        if (e > i + 1) {
            int64_t lo_i = i, hi_i = i;
            for (int64_t j = i + 1; j < e; ++j) {
                if (s[j].a < s[lo_i].a) lo_i = j;
                if (!(s[j].a < s[hi_i].a)) hi_i = j;
            }
            keep = s[lo_i];
            const float fa = s[lo_i].a, ba = s[hi_i].a;
            if (fabs((double)(fa - ba)) > 1e-6) keep.dt = (s[lo_i].phi - s[hi_i].phi) / (fa - ba);
            keep.pad = s[i].pad;
        }
        r[m++] = keep;
        i = e;
    }
    free(it);
    free(s);
    return m;
}

/* ---- the gathers of Input::correct's completion, over the container as it
 * stands: a sorted prefix and the children appended after it, searched with
 * std::upper_bound's loop over the whole range ---- */

/* which records a gather may read: with a wave table, an appended child j is
 * readable once done[j] (the wave that filled it) is below the current wave;
 * reaching one that is not blocks the gather.  Without a table every record
 * is readable (the reference's sequential loop). */
typedef struct {
    const int* done;
    int64_t m;
    int wave;
    int blocked;
} ready_t;

static inline int readable(ready_t* rd, int64_t i)
{
    if (rd->done && i >= rd->m && rd->done[i - rd->m] >= rd->wave) rd->blocked = 1;
    return !rd->blocked;
}

static int64_t afind(const rec48* r, int64_t n, u128 K)
{
    if (n <= 0) return -1;
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count >> 1, it = first + step;
        if (!(K < rkey(&r[it]))) {
            first = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return (first > 0 && key_containing(rkey(&r[first - 1]), K)) ? first - 1 : -1;
}

static inline void afields(const rec48* r, float* f)
{
    f[0] = r->rho; f[1] = r->phi; f[2] = r->dx; f[3] = r->dy; f[4] = r->dz; f[5] = r->a; f[6] = r->dt;
}
static inline void amac(float* acc, const float* f, double w)
{
    for (int q = 0; q < 7; ++q) acc[q] = (float)((double)acc[q] + (double)f[q] * w);
}
static inline void azero(float* a)
{
    for (int q = 0; q < 7; ++q) a[q] = 0.f;
}
static inline double half_of(u128 idx)
{
    return 4.0 / 1.0 * (1.0 / (1.0 * (double)(((u128)1) << key_level(idx)))) / 2.0;
}

/* SimpleHyperOctree::ngp (simplehyperoctree.h:1396-1401) */
static void angp(const rec48* r, int64_t n, double x, double y, double z, float* res, ready_t* rd)
{
    const int64_t f0 = afind(r, n, key_compute(32, x, y, z));
    azero(res);
    if (f0 >= 0 && readable(rd, f0)) afields(&r[f0], res);
}

/* SimpleHyperOctree::cic (simplehyperoctree.h:1410-1469) */
static void acic(const rec48* r, int64_t n, double x, double y, double z, float* res, ready_t* rd)
{
    const double pt[3] = {x, y, z};
    u128 ekey = key_compute(32, x, y, z);
    const int64_t f0 = afind(r, n, ekey);
    u128 idx = (f0 >= 0) ? rkey(&r[f0]) : invalid_key();
    unsigned ilvl = key_level(idx), lvl = ilvl;
    double half = half_of(idx);
    unsigned site = 0;
    azero(res);
    for (int guard = 0; guard <= 33; ++guard) {
        ilvl = lvl;
        if (idx != invalid_key()) {
            double dist[3];
            for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(idx, (unsigned)d) - pt[d]) / (half + half));
            for (unsigned s2 = 0; s2 < 8u; ++s2)
                if (key_containing(key_child(idx, s2), ekey)) {
                    site = s2;
                    break;
                }
            for (unsigned v = 0; v < 8u; ++v) {
                double w = 1.0, vert[3];
                const unsigned diff = site ^ v;
                for (int d = 0; d < 3; ++d) {
                    const int b = (v >> d) & 1u, db = (diff >> d) & 1u;
                    vert[d] = pt[d] + ((double)b * half) - ((double)(!b) * half);
                    w *= ((double)db * (1.0 - dist[d])) + ((double)(!db) * dist[d]);
                }
                ekey = key_compute(ilvl, vert[0], vert[1], vert[2]);
                const int64_t fi = afind(r, n, ekey);
                if (fi >= 0) {
                    if (!readable(rd, fi)) return;
                    const unsigned fl = key_level(rkey(&r[fi]));
                    if (fl < lvl) lvl = fl;
                    float f[7];
                    afields(&r[fi], f);
                    amac(res, f, w);
                } else {
                    azero(res);
                    break;
                }
            }
        }
        if (lvl < ilvl) {
            ekey = key_compute(lvl + 1, x, y, z);
            idx = key_parent(ekey);
            azero(res);
            half = half_of(idx);
        } else {
            break;
        }
    }
}

static inline double tsc_weight(int a, double d)
{
    return (double)a * 0.5 * (1.5 - d) * (1.5 - d) + (double)(1 - a) * (0.75 - d * d);
}

/* SimpleHyperOctree::tsc, uncached (simplehyperoctree.h:1479-1541) */
static void atsc(const rec48* r, int64_t n, double x, double y, double z, float* res, ready_t* rd)
{
    const double pt[3] = {x, y, z};
    u128 ekey = key_compute(32, x, y, z);
    const int64_t f0 = afind(r, n, ekey);
    u128 idx = (f0 >= 0) ? rkey(&r[f0]) : invalid_key();
    unsigned ilvl = key_level(idx), lvl = ilvl;
    double half = half_of(idx);
    azero(res);
    if (x == 0.0 && y == 0.0 && z == 0.0) {
        acic(r, n, 0., 0., 0., res, rd);
        return;
    }
    for (int guard = 0; guard <= 33; ++guard) {
        ilvl = lvl;
        const double tw = 2.0 * half;
        if (idx != invalid_key()) {
            int stop = 0;
            for (int ix = -1; ix <= 1 && !stop; ++ix)
                for (int iy = -1; iy <= 1 && !stop; ++iy)
                    for (int iz = -1; iz <= 1 && !stop; ++iz) {
                        ekey = key_compute(ilvl, pt[0] + ix * tw, pt[1] + iy * tw, pt[2] + iz * tw);
                        const int64_t fi = afind(r, n, ekey);
                        if (fi >= 0) {
                            if (!readable(rd, fi)) return;
                            float f[7];
                            afields(&r[fi], f);
                            double dist[3];
                            for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(ekey, (unsigned)d) - pt[d]) / tw);
                            const double w = tsc_weight(abs(ix), dist[0]) * tsc_weight(abs(iy), dist[1]) *
                                             tsc_weight(abs(iz), dist[2]);
                            const unsigned fl = key_level(rkey(&r[fi]));
                            if (fl < lvl) lvl = fl;
                            if (lvl < ilvl) {
                                azero(res);
                                stop = 1;
                            } else {
                                amac(res, f, w);
                            }
                        } else {
                            azero(res);
                            stop = 1;
                        }
                    }
        }
        if (lvl < ilvl) {
            ekey = key_compute(lvl + 1, x, y, z);
            idx = key_parent(ekey);
            azero(res);
            half = half_of(idx);
        } else {
            break;
        }
    }
}

/* child c of the completion (parent c / 8, site c % 8), gathered over the
 * first m + c records at its centre in float; 0 when the gather is blocked */
static int complete_child(rec48* r, int64_t m, int64_t c, int order, ready_t* rd)
{
    const u128 ck = rkey(&r[m + c]);
    const float cx = (float)key_center(ck, 0), cy = (float)key_center(ck, 1), cz = (float)key_center(ck, 2);
    float f[7];
    if (order == 0) angp(r, m + c, cx, cy, cz, f, rd);
    else if (order == 1) acic(r, m + c, cx, cy, cz, f, rd);
    else atsc(r, m + c, cx, cy, cz, f, rd);
    if (rd->blocked) return 0;
    int empty = 1;
    for (int k = 0; k < 7; ++k) empty = empty && (f[k] == 0.f);
    if (!empty) {
        rec48* o = &r[m + c];
        o->rho = f[0]; o->phi = f[1]; o->dx = f[2]; o->dy = f[3]; o->dz = f[4]; o->a = f[5]; o->dt = f[6];
    }
    return 1;
}

/* non-leaf cells (the next record is a descendant) with a child that find
 * does not resolve (input.h:1451-1458) */
static int incomplete(const rec48* r, int64_t n, int64_t i)
{
    if (i + 1 >= n) return 0;
    const int L = r[i].pad, Ln = r[i + 1].pad;
    if (Ln <= L) return 0;
    uint64_t c[3], cn[3];
    coords_of_key(rkey(&r[i]), L, c);
    coords_of_key(rkey(&r[i + 1]), Ln, cn);
    const int s = Ln - L;
    if ((cn[0] >> s) != c[0] || (cn[1] >> s) != c[1] || (cn[2] >> s) != c[2]) return 0;
    for (int site = 0; site < 8; ++site) {
        const u128 ck = key_of_coords(L + 1, 2 * c[0] + (site & 1), 2 * c[1] + ((site >> 1) & 1), 2 * c[2] + ((site >> 2) & 1));
        if (find_containing(r, n, ck, L + 1) < 0) return 1;
    }
    return 0;
}

/* SimpleHyperOctree::coarsen of the marked cells, then update's removal of
 * the invalidated ones: a cell goes when a strict ancestor is marked */
static int kept_after_coarsen(const rec48* r, int64_t n, const int* mark, int ncoarse, int64_t i)
{
    const int L = r[i].pad;
    uint64_t c[3];
    coords_of_key(rkey(&r[i]), L, c);
    for (int La = L - 1; La >= ncoarse; --La) {
        const int s = L - La;
        const int64_t j = find_containing(r, n, key_of_coords(La, c[0] >> s, c[1] >> s, c[2] >> s), La);
        if (j >= 0 && r[j].pad == La && mark[j]) return 0;
    }
    return 1;
}

static int64_t compact(rec48* r, int64_t n, const int* keep)
{
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i)
        if (keep[i]) r[m++] = r[i];
    return m;
}

/* Utility::interpolate over float tables */
static float interpolate_f(float x0, const float* x, const float* y, int64_t n)
{
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count >> 1, it = first + step;
        if (!(x0 < x[it])) {
            first = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    int64_t i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    return (n > 1) ? (y[i - 1] + ((y[i] - y[i - 1]) * (x0 - x[i - 1]) / (x[i] - x[i - 1]))) : ((n > 0) ? y[0] : 0.f);
}

/* Utility::differentiate<1>, neighbourhood 1: nine-point forward weights of
 * Fornberg's method, step = the abscissae's spacing at x0, in float */
static float forward_derivative_f(float x0, const float* x, const float* y, int64_t n)
{
    const float w[9] = {-761.f / 280.f, 8.f, -14.f, 56.f / 3.f, -35.f / 2.f, 56.f / 5.f, -14.f / 3.f, 8.f / 7.f, -1.f / 8.f};
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count >> 1, it = first + step;
        if (!(x0 < x[it])) {
            first = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    const int64_t j = first + ((n > 1) * ((first <= 0) - (first >= n)));
    const float h = (n > 1) ? ((x[j] - x[j - 1]) * 1u) : 0.f;
    float result = 0.f;
    if (n > 1)
        for (int k = 0; k < 9; ++k) result += w[8 - k] * interpolate_f(x0 + (float)(8 - k) * h, x, y, n);
    return result / h;
}

static int by_float(const void* a, const void* b)
{
    const float x = *(const float*)a, y = *(const float*)b;
    return (x < y) ? -1 : (x > y);
}

/* acorrection (input.h:1485-1506) over the container as it stands: the
 * sorted table of the distinct normal, non-negative scale factors, one
 * shell below it extrapolated against the table's index when that gives a
 * positive normal value below the first, then every cell's a snapped to the
 * table value below it (a cell at the table's first value, or with a value
 * the table dropped, keeps its a: the reference reads before the table
 * there).  Returns -1 without memory. */
static int acorrect(rec48* r, int64_t n, double* amin)
{
    if (n <= 0) return 0;
    float* t = (float*)malloc((size_t)(n + 1) * sizeof(float));
    float* idx = (float*)malloc((size_t)(n + 1) * sizeof(float));
    if (!t || !idx) {
        free(t);
        free(idx);
        return -1;
    }
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        if (!signbit(r[i].a) && normal_f(r[i].a)) t[k++] = r[i].a;
    qsort(t, (size_t)k, sizeof(float), by_float);
    int64_t T = 0;
    for (int64_t i = 0; i < k; ++i)
        if (i == 0 || t[i] != t[i - 1]) t[T++] = t[i];
    if (T > 1) {
        for (int64_t q = 0; q < T; ++q) idx[q] = (float)(q + 1);
        const float below = t[0] - forward_derivative_f(0.f, idx, t, T);
        if (!signbit(below) && isnormal(below) && below < t[0]) {
            memmove(t + 1, t, (size_t)T * sizeof(float));
            t[0] = below;
            ++T;
        }
    }
    if (T > 0) {
        for (int64_t i = 0; i < n; ++i) {
            const float a = r[i].a;
            int64_t lo = 0, hi = T;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (t[mid] < a) lo = mid + 1;
                else hi = mid;
            }
            if (lo > 0) r[i].a = t[lo - 1];
        }
        if (amin) *amin = (double)t[0];
    }
    free(t);
    free(idx);
    return 0;
}

/* Utility::interpolate2 (utility.h:461-468): table in descending order,
 * float result */
static float interpolate2(float x0, const double* x, const double* y, int64_t n)
{
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count >> 1, it = first + step;
        if (!((double)x0 > x[it])) {
            first = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    int64_t i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n > 1) return (float)(y[i - 1] + ((y[i] - y[i - 1]) * ((double)x0 - x[i - 1]) / (x[i] - x[i - 1])));
    return (n > 0) ? (float)y[0] : 0.f;
}

int64_t mpfo_cells_parse(const char* text, int64_t length, float* rows, int64_t capacity)
{
    /* stream >> unsigned >> 9 floats, whitespace separated */
    char* buf = (char*)malloc((size_t)length + 1);
    if (!buf) return -2;
    memcpy(buf, text, (size_t)length);
    buf[length] = 0;
    const char* p = buf;
    char* end = NULL;
    int64_t k = 0;
    for (;;) {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
        if (!*p) break;
        float v[10];
        const unsigned long lv = strtoul(p, &end, 10);
        if (end == p) {
            free(buf);
            return -1;
        }
        p = end;
        v[0] = (float)lv;
        for (int q = 1; q < 10; ++q) {
            v[q] = strtof(p, &end);
            if (end == p) {
                free(buf);
                return -1;
            }
            p = end;
        }
        if (k < capacity)
            for (int q = 0; q < 10; ++q) rows[10 * k + q] = v[q];
        ++k;
    }
    free(buf);
    return k;
}

int64_t mpfo_cells_build(const float* rows, int64_t n, const mpfo_cells_params* P, const mpfo_cosmo* C, void* records,
                         int64_t capacity, double* amin, int64_t* info)
{
    if (n < 0 || !P || !C || P->order < 0 || P->order > 2) return -1;
    if (info)
        for (int q = 0; q < 4; ++q) info[q] = 0;
    if (n == 0) return 0;
    rec48* r = (rec48*)malloc((size_t)n * sizeof(rec48));
    int* keep = (int*)malloc((size_t)(n + 1) * sizeof(int));
    if (!r || !keep) {
        free(r);
        free(keep);
        return -2;
    }
    /* importascii: the file level + log2 EXTENT, the narrow cone's rotation,
       the key of the float position, the cone / sphere filter (file order) */
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        const float* w = rows + 10 * i;
        const int L = (int)(unsigned)w[0] + LEVEL_SHIFT;
        float c[3] = {w[1], w[2], w[3]}, f[3] = {w[6], w[7], w[8]};
        if (P->rotm1) {
            const float ct[3] = {c[0], c[1], c[2]}, ft[3] = {f[0], f[1], f[2]};
            for (int q = 0; q < 3; ++q) {
                const double* R = P->rotm1 + 3 * q;
                c[q] = (float)((double)ct[0] * R[0] + (double)ct[1] * R[1] + (double)ct[2] * R[2]);
                f[q] = (float)((double)ft[0] * R[0] + (double)ft[1] * R[1] + (double)ft[2] * R[2]);
            }
        }
        const u128 k = key_of_coords(L, axis_coord_f(L, c[0]), axis_coord_f(L, c[1]), axis_coord_f(L, c[2]));
        const double pos[3] = {key_center(k, 0), key_center(k, 1), key_center(k, 2)};
        if (!collide(P, L, pos)) continue;
        rec48 o;
        o.lo = (uint64_t)k;
        o.hi = (uint64_t)(k >> 64);
        o.dt = 0.f; o.a = w[9]; o.dx = f[0]; o.dy = f[1]; o.dz = f[2]; o.phi = w[5]; o.rho = w[4];
        o.pad = L;
        r[m++] = o;
    }
    if (P->coarseonly) {
        int64_t q = 0;
        for (int64_t i = 0; i < m; ++i)
            if (r[i].pad == P->ncoarse + LEVEL_SHIFT) r[q++] = r[i];
        m = q;
    }
    if (m <= 0) {
        free(r);
        free(keep);
        return 0;
    }
    /* sistemize (RAMSES units to SI), dphidt = 0, update */
    for (int64_t i = 0; i < m; ++i) {
        const double a = (double)r[i].a;
        const double t = (a * a * P->mpc) / (P->h * 100 * 1000);
        const double l = (a * P->lboxmpch * P->mpc) / P->h;
        r[i].phi = (float)((double)r[i].phi * ((l * l) / (t * t)));
        const double g = (l / (t * t)) * (-a);
        r[i].dx = (float)((double)r[i].dx * g);
        r[i].dy = (float)((double)r[i].dy * g);
        r[i].dz = (float)((double)r[i].dz * g);
        r[i].dt = 0.f;
    }
    int64_t status = 0;
    m = update(r, m);
    int ncoarse = 64, nmax = 0;
    for (int64_t i = 0; i < m; ++i) {
        ncoarse = r[i].pad < ncoarse ? r[i].pad : ncoarse;
        nmax = r[i].pad > nmax ? r[i].pad : nmax;
    }
    int* mark = (int*)calloc((size_t)m + 1, sizeof(int));
    float* rho0 = (float*)malloc((size_t)m * sizeof(float) + 1);
    if (m < 0 || !mark || !rho0) {
        status = -2;
        goto done;
    }
    /* Input::correct: coarse cells with a non-normal density take the mean of
       their same-level neighbours with a normal one (densities before any
       correction) */
    if (P->coarsecorrection) {
        for (int64_t i = 0; i < m; ++i) rho0[i] = r[i].rho;
        for (int64_t i = 0; i < m; ++i) {
            if (r[i].pad != ncoarse || normal_f(rho0[i])) continue;
            const int L = ncoarse;
            uint64_t c[3];
            coords_of_key(rkey(&r[i]), L, c);
            const uint64_t mask = (L >= 64) ? ~0ULL : ((1ULL << L) - 1ULL);
            float result = 0.f;
            unsigned count = 0;
            for (int ix = -1; ix <= 1; ++ix)
                for (int iy = -1; iy <= 1; ++iy)
                    for (int iz = -1; iz <= 1; ++iz) {
                        if (ix == 0 && iy == 0 && iz == 0) continue;
                        const u128 nk = key_of_coords(L, (c[0] + (uint64_t)(int64_t)ix) & mask,
                                                      (c[1] + (uint64_t)(int64_t)iy) & mask,
                                                      (c[2] + (uint64_t)(int64_t)iz) & mask);
                        const int64_t j = find_containing(r, m, nk, L);
                        if (j >= 0 && normal_f(rho0[j])) {
                            result += rho0[j];
                            ++count;
                        }
                    }
            r[i].rho = result / (float)(count + (count == 0));
        }
    }
    int64_t ninc = 0;
    if (!P->correction) {
        /* the parents of refined cells with a non-normal density coarsened,
           then the incomplete octs coarsened too; the invalidated cells stay
           in the container (for acorrection) until the final update */
        for (int64_t i = 0; i < m; ++i) {
            const int L = r[i].pad;
            if (L <= ncoarse || normal_f(r[i].rho)) continue;
            uint64_t c[3];
            coords_of_key(rkey(&r[i]), L, c);
            const int64_t p = find_containing(r, m, key_of_coords(L - 1, c[0] >> 1, c[1] >> 1, c[2] >> 1), L - 1);
            if (p >= 0) mark[p] = 1;
        }
        for (int64_t i = 0; i < m; ++i) keep[i] = kept_after_coarsen(r, m, mark, ncoarse, i);
        m = compact(r, m, keep);
        for (int64_t i = 0; i < m; ++i) mark[i] = incomplete(r, m, i);
        for (int64_t i = 0; i < m; ++i) keep[i] = kept_after_coarsen(r, m, mark, ncoarse, i);
        if (P->acorrection && acorrect(r, m, amin) != 0) {
            status = -2;
            goto done;
        }
        m = compact(r, m, keep);
    } else {
        /* refined cells whose dphidt, then rho, is not normal take the
           parent's, level by level (parents before children) */
        for (int which = 0; which < 2; ++which)
            for (int L = ncoarse + 1; L <= nmax; ++L)
                for (int64_t i = 0; i < m; ++i) {
                    if (r[i].pad != L) continue;
                    const float v = which ? r[i].rho : r[i].dt;
                    if (normal_f(v)) continue;
                    uint64_t c[3];
                    coords_of_key(rkey(&r[i]), L, c);
                    const int64_t p = find_containing(r, m, key_of_coords(L - 1, c[0] >> 1, c[1] >> 1, c[2] >> 1), L - 1);
                    if (p < 0) continue;
                    if (which) r[i].rho = r[p].rho;
                    else r[i].dt = r[p].dt;
                }
        for (int64_t i = 0; i < m; ++i) ninc += incomplete(r, m, i);
    }
    if (ninc > 0) {
        /* the children of each incomplete cell (key order) appended and
           gathered at their centres over the container so far */
        const int64_t nch = 8 * ninc;
        rec48* g = (rec48*)realloc(r, (size_t)(m + nch) * sizeof(rec48));
        int* done = (int*)malloc((size_t)nch * sizeof(int));
        if (!g || !done) {
            if (g) r = g;
            free(done);
            status = -2;
            goto done;
        }
        r = g;
        int64_t c = 0;
        for (int64_t i = 0; i < m; ++i) {
            if (!incomplete(r, m, i)) continue;
            for (unsigned site = 0; site < 8; ++site, ++c) {
                rec48 o = r[i];
                const u128 ck = key_child(rkey(&r[i]), site);
                o.lo = (uint64_t)ck;
                o.hi = (uint64_t)(ck >> 64);
                o.pad = r[i].pad + 1;
                r[m + c] = o;
                done[c] = INT32_MAX;
            }
        }
        /* the reference's loop fills child after child; with completion_waves
           = k > 0 the children are filled as the device does, in at most k
           waves of gathers that read only children of earlier waves, and the
           rest in order after them */
        int wave = 0;
        int64_t left = nch;
        while (left > 0 && wave < P->completion_waves) {
            ++wave;
            left = 0;
            for (int64_t q = 0; q < nch; ++q) {
                if (done[q] != INT32_MAX) continue;
                ready_t rd = {done, m, wave, 0};
                if (complete_child(r, m, q, P->order, &rd)) done[q] = wave;
                else ++left;
            }
        }
        for (int64_t q = 0; q < nch && left > 0; ++q) {
            if (done[q] != INT32_MAX) continue;
            ready_t rd = {NULL, m, 0, 0};
            complete_child(r, m, q, P->order, &rd);
        }
        if (info) {
            info[0] = ninc;
            info[1] = nch - left;
            info[2] = wave;
            info[3] = left;
        }
        free(done);
        if (P->acorrection && acorrect(r, m + nch, amin) != 0) {
            status = -2;
            goto done;
        }
        m = update(r, m + nch);
        if (m < 0) {
            status = -2;
            goto done;
        }
    } else if (P->correction && P->acorrection && acorrect(r, m, amin) != 0) {
        status = -2;
        goto done;
    }
    /* correctOctree: dphidt *= da/dt at the cell's a */
    for (int64_t i = 0; i < m; ++i) {
        r[i].dt *= interpolate2(r[i].a, C->a, C->dadt, C->n);
        r[i].pad = 0;
    }
    if (records) memcpy(records, r, (size_t)(m < capacity ? m : capacity) * sizeof(rec48));
    status = m;
done:
    free(r);
    free(keep);
    free(mark);
    free(rho0);
    return status;
}
