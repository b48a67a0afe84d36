/* CPU oracle: plain-C restatement of the reference photon-propagation path.
 * TEST INFRASTRUCTURE ONLY (see mpf_oracle.h).  Build with -ffp-contract=off.
 *
 * Sources restated (reference paths):
 *   keys             src/magrathea/simplehyperoctreeindex.h:572-575 (level),
 *                    :679-694 (parent/child), :888-893 (center),
 *                    :950-955 (extent), :997-1001 (containing),
 *                    :1165-1189 (compute/cipher)
 *   locate           src/magrathea/simplehyperoctree.h:874-899
 *   cic              src/magrathea/simplehyperoctree.h:1410-1469
 *   tsc (cached)     src/magrathea/simplehyperoctree.h:1552-1644
 *   mac              src/magrathea/simplehyperoctree.h:1905-1910
 *   interpolate      src/utility.h:441-449
 *   launch (6 args)  src/integrator.h:283-309
 *   dphotondl        src/integrator.h:409-445
 *   integrate (stop) src/integrator.h:648-824
 *   Jacobian         src/lensing.h:399-472
 *   plane crossings  src/hmaps.h:612-676 (per-surface interpolation)
 */
#include "mpf_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "mpf_oracle_keys.h"

static const double C_LIGHT = 299792458.0;

static inline u128 tkey(const mpfo_tree* T, int64_t i) { return mk(T->keys[2 * i], T->keys[2 * i + 1]); }

/* Number of keys <= K (std::upper_bound position). */
static inline int64_t upper(const mpfo_tree* T, u128 K)
{
    int64_t first = 0, count = T->n;
    while (count > 0) {
        const int64_t step = count / 2, it = first + step;
        if (!(K < tkey(T, it))) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return first;
}

/* The reference's lookup: the last key <= K if it contains K, else -1. */
static inline int64_t find(const mpfo_tree* T, u128 K)
{
    if (T->n <= 0) return -1;
    const int64_t m = upper(T, K);
    return (m > 0 && key_containing(tkey(T, m - 1), K)) ? m - 1 : -1;
}

int64_t mpfo_locate(const mpfo_tree* T, double x, double y, double z)
{
    return find(T, key_compute(32, x, y, z));
}

/* SimpleHyperOctree::ngp (simplehyperoctree.h:1396-1401): the record of the
   cell found for the position's level-32 key, or the empty record */
/* A cell's record as the gathers read it: the 7 fields, then the velocity
   slots of a velocity-field octree (gravity2.h:45; zeros without one). */
#define NF 10
static inline void load_rec(const mpfo_tree* T, int64_t i, float* f)
{
    for (int k = 0; k < 7; ++k) f[k] = T->fields[7 * i + k];
    for (int k = 0; k < 3; ++k) f[7 + k] = T->vel ? T->vel->v[3 * i + k] : 0.0f;
}

static void ngp10(const mpfo_tree* T, double x, double y, double z, float* res)
{
    const int64_t i = find(T, key_compute(32, x, y, z));
    if (i >= 0) load_rec(T, i, res);
    else for (int k = 0; k < NF; ++k) res[k] = 0.0f;
}

void mpfo_ngp(const mpfo_tree* T, double x, double y, double z, float* res)
{
    float r[NF];
    ngp10(T, x, y, z, r);
    memcpy(res, r, 7 * sizeof(float));
}

void mpfo_key_compute(unsigned level, double x, double y, double z, uint64_t* out)
{
    const u128 k = key_compute(level, x, y, z);
    out[0] = (uint64_t)(k >> 64);
    out[1] = (uint64_t)k;
}

unsigned mpfo_key_level(uint64_t hi, uint64_t lo) { return key_level(mk(hi, lo)); }

/* the reference's multiply-accumulate of every arithmetic member
   (simplehyperoctree.h:1887-1910): float += float * double; the velocity
   slots only when the octree has them */
static inline void mac(const mpfo_tree* T, float* acc, const float* f, double w)
{
    const int nf = T->vel ? NF : 7;
    for (int k = 0; k < nf; ++k) acc[k] = (float)((double)acc[k] + (double)f[k] * w);
}

static inline void zero7(float* a) { for (int k = 0; k < NF; ++k) a[k] = 0.0f; }

/* data == empty: every member zero, the velocity slots included */
static inline int empty7(const float* a)
{
    for (int k = 0; k < NF; ++k) if (a[k] != 0.0f) return 0;
    return 1;
}

static void cic10(const mpfo_tree* T, double x, double y, double z, float* res)
{
    const double pt[3] = {x, y, z};
    u128 ekey = key_compute(32, x, y, z);
    const int64_t f0 = find(T, ekey);
    u128 idx = (f0 >= 0) ? tkey(T, f0) : invalid_key();
    unsigned ilvl = key_level(idx), lvl = ilvl;
    double half = (double)OCT_EXTENT / 1.0 * key_extent1(idx) / 2.0;
    unsigned site = 0;
    zero7(res);
    do {
        ilvl = lvl;
        if (idx != invalid_key()) {
            double dist[3];
            for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(idx, d) - pt[d]) / (half + half));
            for (unsigned s = 0; s < 8u; ++s)
                if (key_containing(key_child(idx, s), ekey)) { site = s; break; }
            for (unsigned v = 0; v < 8u; ++v) {
                double w = 1.0, vert[3];
                const unsigned diff = site ^ v;
                for (int d = 0; d < 3; ++d) {
                    const int b = (v >> d) & 1u, db = (diff >> d) & 1u;
                    vert[d] = pt[d] + ((double)b * half) - ((double)(!b) * half);
                    w *= ((double)db * (1.0 - dist[d])) + ((double)(!db) * dist[d]);
                }
                ekey = key_compute(ilvl, vert[0], vert[1], vert[2]);
                const int64_t fi = find(T, ekey);
                if (fi >= 0) {
                    const unsigned fl = key_level(tkey(T, fi));
                    if (fl < lvl) lvl = fl;
                    float f[NF];
                    load_rec(T, fi, f);
                    mac(T, res, f, w);
                } else {
                    zero7(res);
                    break;
                }
            }
        }
        if (lvl < ilvl) {
            ekey = key_compute(lvl + 1, x, y, z);
            idx = key_parent(ekey);
            zero7(res);
            half = (double)OCT_EXTENT / 1.0 * key_extent1(idx) / 2.0;
        }
    } while (lvl < ilvl);
}

void mpfo_cic(const mpfo_tree* T, double x, double y, double z, float* res)
{
    float r[NF];
    cic10(T, x, y, z, r);
    memcpy(res, r, 7 * sizeof(float));
}

typedef struct {
    u128 key[27];
    float f[27][NF];
} tsc_cache;

static inline void cache_init(tsc_cache* c) { memset(c, 0, sizeof(*c)); }

static inline double tsc_w(int a, double d)
{
    return (double)a * 0.5 * (1.5 - d) * (1.5 - d) + (double)(1 - a) * (0.75 - d * d);
}

static void tsc_cached(const mpfo_tree* T, tsc_cache* cache, double x, double y, double z, float* res)
{
    const double pt[3] = {x, y, z};
    u128 ekey = key_compute(32, x, y, z);
    const int64_t f0 = find(T, ekey);
    u128 idx = (f0 >= 0) ? tkey(T, f0) : invalid_key();
    unsigned ilvl = key_level(idx), lvl = ilvl;
    double half = (double)OCT_EXTENT / 1.0 * key_extent1(idx) / 2.0;
    zero7(res);
    if (x == 0.0 && y == 0.0 && z == 0.0) {
        cic10(T, 0., 0., 0., res);
        return;
    }
    tsc_cache tmp;
    do {
        ilvl = lvl;
        const double tw = 2.0 * half;
        if (cache->key[13] == idx) {
            int ic = 0;
            for (int ix = -1; ix <= 1; ++ix)
                for (int iy = -1; iy <= 1; ++iy)
                    for (int iz = -1; iz <= 1; ++iz) {
                        double dist[3];
                        for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(cache->key[ic], d) - pt[d]) / tw);
                        const double w = tsc_w(abs(ix), dist[0]) * tsc_w(abs(iy), dist[1]) * tsc_w(abs(iz), dist[2]);
                        mac(T, res, cache->f[ic], w);
                        ++ic;
                    }
            return;
        } else if (idx != invalid_key()) {
            int ic = 0, stop = 0;
            for (int ix = -1; ix <= 1 && !stop; ++ix)
                for (int iy = -1; iy <= 1 && !stop; ++iy)
                    for (int iz = -1; iz <= 1 && !stop; ++iz) {
                        ekey = key_compute(ilvl, pt[0] + ix * tw, pt[1] + iy * tw, pt[2] + iz * tw);
                        const int64_t fi = find(T, ekey);
                        if (fi >= 0) {
                            tmp.key[ic] = tkey(T, fi);
                            load_rec(T, fi, tmp.f[ic]);
                            double dist[3];
                            for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(ekey, d) - pt[d]) / tw);
                            const double w = tsc_w(abs(ix), dist[0]) * tsc_w(abs(iy), dist[1]) * tsc_w(abs(iz), dist[2]);
                            const unsigned fl = key_level(tmp.key[ic]);
                            if (fl < lvl) lvl = fl;
                            if (lvl < ilvl) { zero7(res); stop = 1; }
                            else { mac(T, res, tmp.f[ic], w); ++ic; }
                        } else {
                            zero7(res);
                            stop = 1;
                        }
                    }
            if (ic == 27) *cache = tmp;
        }
        if (lvl < ilvl) {
            ekey = key_compute(lvl + 1, x, y, z);
            idx = key_parent(ekey);
            zero7(res);
            half = (double)OCT_EXTENT / 1.0 * key_extent1(idx) / 2.0;
        }
    } while (lvl < ilvl);
}

void mpfo_tsc(const mpfo_tree* T, double x, double y, double z, float* out)
{
    tsc_cache c;
    cache_init(&c);
    float r[NF];
    tsc_cached(T, &c, x, y, z, r);
    memcpy(out, r, 7 * sizeof(float));
}

double mpfo_interpolate(double x0, const double* x, const double* y, int64_t n)
{
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count / 2, it = first + step;
        if (!(x0 < x[it])) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    int64_t i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    return (n > 1) ? (y[i - 1] + ((y[i] - y[i - 1]) * (x0 - x[i - 1]) / (x[i] - x[i - 1]))) : ((n > 0) ? y[0] : 0.0);
}

/* ---------------------------------------------------------------------- */
/* integrator                                                              */
/* ---------------------------------------------------------------------- */
enum { PA = 0, PT, PX, PY, PZ, PK0, PK1, PK2, PK3, PLEVEL, PAH, PRHO, PPHI, PDX, PDY, PDZ, PDT, PDL, PLAP, PZRED,
       PDS2, PERR, PISW, PISWOLD, PCHI, PLAMBDA, PS, PINDEX };

typedef struct {
    const mpfo_tree* T;
    const mpfo_cosmo* C;
    int order;
    double length;
    tsc_cache cache;
    int homogeneous;   /* Order = -1 (integrator.h:425, 676, 744): the homogeneous field, the octree's levels */
} ctx_t;

static inline void gather(ctx_t* c, double x, double y, double z, float* d)
{
    if (c->homogeneous) {   /* a = 1, the rest 0; dphotondl reads only the zero gradient and dphidt */
        zero7(d);
        d[5] = 1.0f;   /* a, the record order rho phi dx dy dz a dt */
        return;
    }
    if (c->order == 0) ngp10(c->T, x, y, z, d);
    else if (c->order == 1) cic10(c->T, x, y, z, d);
    else tsc_cached(c->T, &c->cache, x, y, z, d);
}

/* field indices in the record: the 7 fields, then the velocity slots */
enum { FRHO = 0, FPHI, FDX, FDY, FDZ, FA, FDT, FVX, FVY, FVZ };

static void dphotondl(ctx_t* c, double* out, const double* in)
{
    const double two = 2.0;
    const double c2 = C_LIGHT * C_LIGHT;
    float d[NF];
    gather(c, in[PX], in[PY], in[PZ], d);
    const double dphidl = (double)d[FDT] * in[PK0] + ((double)d[FDX] * in[PK1] + (double)d[FDY] * in[PK2] + (double)d[FDZ] * in[PK3]);
    const double dadt = mpfo_interpolate(in[PT], c->C->t, c->C->dadt, c->C->n);
    const double scale = c->length;
    out[PA] = in[PK0] * dadt;
    out[PT] = in[PK0];
    out[PX] = in[PK1] / scale;
    out[PY] = in[PK2] / scale;
    out[PZ] = in[PK3] / scale;
    out[PK0] = -(two * dadt / in[PA] * in[PK0] * in[PK0]) - (two / c2 * in[PK0]) * (dphidl - (double)d[FDT] * in[PK0]);
    out[PK1] = -(two * dadt / in[PA] * in[PK0] * in[PK1]) + (two / c2 * dphidl * in[PK1]) - (two * (double)d[FDX] * in[PK0] * in[PK0]);
    out[PK2] = -(two * dadt / in[PA] * in[PK0] * in[PK2]) + (two / c2 * dphidl * in[PK2]) - (two * (double)d[FDY] * in[PK0] * in[PK0]);
    out[PK3] = -(two * dadt / in[PA] * in[PK0] * in[PK3]) + (two / c2 * dphidl * in[PK3]) - (two * (double)d[FDZ] * in[PK0] * in[PK0]);
}

typedef struct {
    double* p;
    int64_t n, cap;
} traj_t;

static double* traj_push(traj_t* t)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 256;
        t->p = (double*)realloc(t->p, (size_t)t->cap * MPFO_PHOTON * sizeof(double));
    }
    return t->p + MPFO_PHOTON * (t->n++);
}

static int stop_reached(int kind, double ref, const double* back, const double* photon, const double* ki)
{
    switch (kind) {
    case MPFO_STOP_R: return back[PCHI] > ref;
    case MPFO_STOP_LAMBDA: return back[PLAMBDA] > ref;
    case MPFO_STOP_REDSHIFT: return back[PZRED] > ref;
    case MPFO_STOP_T: return back[PT] > ref;
    case MPFO_STOP_A: return back[PA] < ref;
    case MPFO_STOP_PLANE: return (photon[PX] * ki[0] + photon[PY] * ki[1] + photon[PZ] * ki[2]) > ref;
    case MPFO_STOP_S: return back[PS] > ref;
    default: return 1;
    }
}

/* integrate() with a stop criterion; the trajectory grows in *tr. */
static void integrate(ctx_t* c, traj_t* tr, unsigned nsteps, int stop_kind, double stop_ref, const double* ki)
{
    const double zero = 0.0, one = 1.0, two = 2.0, six = 6.0;
    const double cl = C_LIGHT, c2 = C_LIGHT * C_LIGHT;
    const double mn = 0.0 - (double)OCT_EXTENT / two, mx = 0.0 + (double)OCT_EXTENT / two;
    const double scale = c->length;
    float data[NF];
    double* b = tr->p + MPFO_PHOTON * (tr->n - 1);
    gather(c, b[PX], b[PY], b[PZ], data);
    const double norm = sqrt((c2 * (one + two * ((double)data[FPHI] / c2)) * b[PK0] * b[PK0]) /
                             ((one - two * ((double)data[FPHI] / c2)) * (b[PK1] * b[PK1] + b[PK2] * b[PK2] + b[PK3] * b[PK3])));
    b[PK1] *= norm;
    b[PK2] *= norm;
    b[PK3] *= norm;
    b[PA] = mpfo_interpolate(b[PT], c->C->t, c->C->a, c->C->n);
    int64_t loc = mpfo_locate(c->T, b[PX], b[PY], b[PZ]);
    b[PLEVEL] = (loc >= 0) ? (double)key_level(tkey(c->T, loc)) : 0.0;
    b[PAH] = zero;
    b[PRHO] = data[FRHO];
    b[PPHI] = data[FPHI];
    b[PDX] = data[FDX];
    b[PDY] = data[FDY];
    b[PDZ] = data[FDZ];
    b[PDT] = data[FDT];
    b[PDL] = zero;
    b[PLAP] = zero;
    b[PZRED] = zero;
    b[PDS2] = (b[PA] * b[PA]) * (-(c2 * (one + two * (b[PPHI] / c2)) * b[PK0] * b[PK0]) +
                                 ((one - two * (b[PPHI] / c2)) * (b[PK1] * b[PK1] + b[PK2] * b[PK2] + b[PK3] * b[PK3])));
    b[PERR] = one - ((one - two * (b[PPHI] / c2)) * (b[PK1] * b[PK1] + b[PK2] * b[PK2] + b[PK3] * b[PK3])) /
                        (c2 * (one + two * (b[PPHI] / c2)) * b[PK0] * b[PK0]);
    b[PISW] = zero;
    b[PCHI] = zero;
    b[PISWOLD] = zero;
    b[PLAMBDA] = zero;
    b[PS] = zero;
    double ratio = b[PA] * b[PA] * (scale / cl) / nsteps;
    double dl = (loc >= 0 ? key_extent4(tkey(c->T, loc)) : 0.0) * ratio;
    const double a0 = b[PA];
    /* velocity-field octree: the observer velocity along trajectory[0]'s
       direction (integrator.h:707-708) */
    const mpfo_velocity* vf = c->T->vel;
    const double* t0 = tr->p;
    const double v0n = vf ? (vf->vobs[0] * t0[PK1] + vf->vobs[1] * t0[PK2] + vf->vobs[2] * t0[PK3]) / (cl * t0[PK0]) : 0.0;
    const double phi0c2 = b[PPHI] / c2;
    double photon[MPFO_PHOTON];
    memset(photon, 0, sizeof(photon));
    double dcore[4][9];
    while (!empty7(data)) {
        b = tr->p + MPFO_PHOTON * (tr->n - 1);
        photon[PINDEX] = b[PINDEX] + one;
        dphotondl(c, dcore[0], b);
        for (int i = 0; i < 9; ++i) photon[i] = b[i] + dl / two * dcore[0][i];
        dphotondl(c, dcore[1], photon);
        for (int i = 0; i < 9; ++i) photon[i] = b[i] + dl / two * dcore[1][i];
        dphotondl(c, dcore[2], photon);
        for (int i = 0; i < 9; ++i) photon[i] = b[i] + dl * dcore[2][i];
        dphotondl(c, dcore[3], photon);
        for (int i = 0; i < 9; ++i)
            photon[i] = b[i] + (dl / six) * (dcore[0][i] + two * dcore[1][i] + two * dcore[2][i] + dcore[3][i]);
        gather(c, photon[PX], photon[PY], photon[PZ], data);
        if (!(!(photon[PA] < zero) && ((photon[PX] > mn) && (photon[PX] < mx) && (photon[PY] > mn) &&
                                       (photon[PY] < mx) && (photon[PZ] > mn) && (photon[PZ] < mx))))
            zero7(data);
        loc = mpfo_locate(c->T, photon[PX], photon[PY], photon[PZ]);
        photon[PLEVEL] = (loc >= 0) ? (double)key_level(tkey(c->T, loc)) : 0.0;
        photon[PAH] = data[FA];
        photon[PRHO] = data[FRHO];
        photon[PPHI] = data[FPHI];
        photon[PDX] = data[FDX];
        photon[PDY] = data[FDY];
        photon[PDZ] = data[FDZ];
        photon[PDT] = -(double)data[FDT];
        photon[PDL] = (double)data[FDT] * photon[PK0] + (photon[PDX] * photon[PK1] + photon[PDY] * photon[PK2] + photon[PDZ] * photon[PK3]);
        photon[PLAP] = ((double)data[FPHI] - b[PPHI]) / dl;
        photon[PDS2] = (photon[PA] * photon[PA]) * ((-c2 * (one + two * (photon[PPHI] / c2)) * photon[PK0] * photon[PK0]) +
                                                    ((one - two * (photon[PPHI] / c2)) * (photon[PK1] * photon[PK1] + photon[PK2] * photon[PK2] + photon[PK3] * photon[PK3])));
        photon[PERR] = one - ((one - two * (photon[PPHI] / c2)) * (photon[PK1] * photon[PK1] + photon[PK2] * photon[PK2] + photon[PK3] * photon[PK3])) /
                                 (c2 * (one + two * (photon[PPHI] / c2)) * photon[PK0] * photon[PK0]);
        photon[PISW] += (b[PDT] + photon[PDT]) * (photon[PT] - b[PT]) / c2;
        photon[PISWOLD] -= 2 * (photon[PPHI] - b[PPHI]) / c2 -
                           ((b[PDX] + photon[PDX]) * (photon[PX] - b[PX]) * scale + (b[PDY] + photon[PDY]) * (photon[PY] - b[PY]) * scale +
                            (b[PDZ] + photon[PDZ]) * (photon[PZ] - b[PZ]) * scale) / c2;
        photon[PCHI] = sqrt(photon[PX] * photon[PX] + photon[PY] * photon[PY] + photon[PZ] * photon[PZ]);
        photon[PLAMBDA] += dl;
        photon[PS] += sqrt((photon[PX] - b[PX]) * (photon[PX] - b[PX]) + (photon[PY] - b[PY]) * (photon[PY] - b[PY]) +
                           (photon[PZ] - b[PZ]) * (photon[PZ] - b[PZ]));
        if (vf) /* integrator.h:765-767 */
            photon[PZRED] = a0 / photon[PA] * (one + phi0c2 - photon[PPHI] / c2 + photon[PISW] +
                                               (data[FVX] * photon[PK1] + data[FVY] * photon[PK2] + data[FVZ] * photon[PK3]) /
                                                   (cl * photon[PK0]) - v0n) - one;
        else
            photon[PZRED] = a0 / photon[PA] * (one + phi0c2 - photon[PPHI] / c2) - one;
        if (!empty7(data)) {
            ratio = photon[PA] * photon[PA] * (scale / cl) / nsteps;
            dl = (loc >= 0 ? key_extent4(tkey(c->T, loc)) : 0.0) * ratio;
            double* dst = traj_push(tr);
            memcpy(dst, photon, sizeof(photon));
        }
        b = tr->p + MPFO_PHOTON * (tr->n - 1);
        if (stop_reached(stop_kind, stop_ref, b, photon, ki)) break;
    }
    if (tr->n > 0) {
        b = tr->p + MPFO_PHOTON * (tr->n - 1);
        if (signbit(b[PZRED]) || signbit(b[PA])) tr->n--;
    }
}

static void launch6(const double* L, double* p)
{
    memset(p, 0, MPFO_PHOTON * sizeof(double));
    const double norm = sqrt((L[3] - L[0]) * (L[3] - L[0]) + (L[4] - L[1]) * (L[4] - L[1]) + (L[5] - L[2]) * (L[5] - L[2]));
    p[PA] = 1.0;
    p[PT] = 0.0;
    p[PX] = L[0];
    p[PY] = L[1];
    p[PZ] = L[2];
    p[PK0] = 1.0;
    p[PK1] = (L[3] - L[0]) / norm;
    p[PK2] = (L[4] - L[1]) / norm;
    p[PK3] = (L[5] - L[2]) / norm;
}

/* ---------------------------------------------------------------------- */
/* Jacobian and planes                                                     */
/* ---------------------------------------------------------------------- */
static int64_t upper_by(const traj_t* tr, int q, double v, int descending)
{
    int64_t first = 0, count = tr->n;
    while (count > 0) {
        const int64_t step = count / 2, it = first + step;
        const double e = tr->p[MPFO_PHOTON * it + q];
        const int less = descending ? (v > e) : (v < e);
        if (!less) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return first;
}

static void jacobian(ctx_t* c, const traj_t* tr, int nd, const double* dist, double* A /* nd x 3 */)
{
    const double c2 = C_LIGHT * C_LIGHT;
    double* a11 = (double*)calloc((size_t)nd * (size_t)tr->n, sizeof(double));
    double* a12 = (double*)calloc((size_t)nd * (size_t)tr->n, sizeof(double));
    double* a22 = (double*)calloc((size_t)nd * (size_t)tr->n, sizeof(double));
    tsc_cache cache;
    cache_init(&cache);
    for (int64_t i = 1; i < tr->n; ++i) {
        const double* P = tr->p + MPFO_PHOTON * i;
        const double* Q = tr->p + MPFO_PHOTON * (i - 1);
        const double x = P[PX], y = P[PY], z = P[PZ], r = P[PCHI];
        const double phi = atan2(y, x);
        const double theta = acos(z / r);
        const double cp = cos(phi), sp = sin(phi), ct = cos(theta), st = sin(theta);
        const double s2p = sin(2 * phi), s2t = sin(2 * theta);
        const double dl = pow(2, -(P[PLEVEL] - 1 - LEVEL_SHIFT));
        float xm[NF], xp[NF], ym[NF], yp[NF], zm[NF], zp[NF];
        tsc_cached(c->T, &cache, x - 0.5 * dl, y, z, xm);
        tsc_cached(c->T, &cache, x + 0.5 * dl, y, z, xp);
        tsc_cached(c->T, &cache, x, y - 0.5 * dl, z, ym);
        tsc_cached(c->T, &cache, x, y + 0.5 * dl, z, yp);
        tsc_cached(c->T, &cache, x, y, z - 0.5 * dl, zm);
        tsc_cached(c->T, &cache, x, y, z + 0.5 * dl, zp);
        const double dxxp = (xp[FDX] - xm[FDX]) / dl;
        const double dxyp = (yp[FDX] - ym[FDX]) / dl;
        const double dxzp = (zp[FDX] - zm[FDX]) / dl;
        const double dyyp = (yp[FDY] - ym[FDY]) / dl;
        const double dyzp = (zp[FDY] - zm[FDY]) / dl;
        const double dzzp = (zp[FDZ] - zm[FDZ]) / dl;
        const double d1d1p = sp * sp * dxxp + cp * cp * dyyp - s2p * dxyp;
        const double d2d2p = cp * cp * ct * ct * dxxp + sp * sp * ct * ct * dyyp + st * st * dzzp + s2p * ct * ct * dxyp - sp * s2t * dyzp - cp * s2t * dxzp;
        const double d1d2p = ct * cp * sp * (dyyp - dxxp) + (cp * cp - sp * sp) * ct * dxyp + sp * st * dxzp - cp * st * dyzp;
        const double dr = P[PCHI] - Q[PCHI];
        for (int j = 0; j < nd; ++j) {
            const double gxsx = (dist[j] - P[PCHI]) * P[PCHI] / dist[j];
            const int64_t o = (int64_t)j * tr->n;
            a11[o + i] = a11[o + i - 1] + gxsx * d1d1p * dr;
            a12[o + i] = a12[o + i - 1] + gxsx * d1d2p * dr;
            a22[o + i] = a22[o + i - 1] + gxsx * d2d2p * dr;
        }
    }
    for (int j = 0; j < nd; ++j) {
        const int64_t marked = upper_by(tr, PCHI, dist[j], 0);
        const int64_t fid = marked - (marked > 0);
        const int64_t o = (int64_t)j * tr->n;
        A[3 * j + 0] = 1 - 2 * a11[o + fid] / c2 * c->length;
        A[3 * j + 1] = -2 * a12[o + fid] / c2 * c->length;
        A[3 * j + 2] = 1 - 2 * a22[o + fid] / c2 * c->length;
    }
    free(a11);
    free(a12);
    free(a22);
}

static int stop_quantity(int kind)
{
    switch (kind) {
    case MPFO_STOP_R: return PCHI;
    case MPFO_STOP_LAMBDA: return PLAMBDA;
    case MPFO_STOP_T: return PT;
    case MPFO_STOP_A: return PA;
    case MPFO_STOP_S: return PS;
    case MPFO_STOP_REDSHIFT: return PZRED;
    default: return -1;
    }
}

static void planes_of(ctx_t* c, const traj_t* tr, int stop_kind, int np, const double* planes, int jac, double* out)
{
    const int q = stop_quantity(stop_kind);
    double* dist = (double*)malloc(sizeof(double) * (size_t)(np > 0 ? np : 1));
    for (int i = 0; i < np; ++i) {
        double* o = out + MPFO_PLANE * i;
        memset(o, 0, MPFO_PLANE * sizeof(double));
        int64_t marked;
        if (q < 0 || tr->n == 0) { marked = tr->n; }
        else if (stop_kind == MPFO_STOP_REDSHIFT) {
            marked = tr->n;
            for (int64_t k = 0; k < tr->n; ++k)
                if (tr->p[MPFO_PHOTON * k + PZRED] > planes[i]) { marked = k; break; }
        } else marked = upper_by(tr, q, planes[i], stop_kind == MPFO_STOP_A);
        const int64_t fid = marked - (marked > 0);
        o[0] = (double)fid;
        o[19] = (tr->n > 0 && q >= 0 && fid + 1 < tr->n && !(fid == tr->n - 1 || fid == 0)) ? 1.0 : 0.0;
        dist[i] = 0.0;
        if (!(tr->n > 0 && q >= 0 && fid + 1 < tr->n)) continue;
        const double* P0 = tr->p + MPFO_PHOTON * fid;
        const double* P1 = tr->p + MPFO_PHOTON * (fid + 1);
        const double f = (P1[q] - planes[i]) / (P1[q] - P0[q]);
        o[1] = f;
        o[2] = P0[PX] * f + P1[PX] * (1 - f);
        o[3] = P0[PY] * f + P1[PY] * (1 - f);
        o[4] = P0[PZ] * f + P1[PZ] * (1 - f);
        o[5] = sqrt(o[2] * o[2] + o[3] * o[3] + o[4] * o[4]);
        dist[i] = o[5];
        const int qs[9] = {PT, PA, PZRED, PCHI, PLAMBDA, PS, PISW, PRHO, PPHI};
        for (int k = 0; k < 9; ++k) o[9 + k] = P0[qs[k]] * f + P1[qs[k]] * (1 - f);
        double mx = 0.0;
        int have = 0;
        for (int64_t k = 0; k < fid; ++k) {
            const double r = tr->p[MPFO_PHOTON * k + PRHO];
            if (!have || mx < r) { mx = r; have = 1; }
        }
        o[18] = mx;
    }
    if (jac && np > 0 && tr->n > 0) {
        double* A = (double*)malloc(sizeof(double) * 3 * (size_t)np);
        jacobian(c, tr, np, dist, A);
        for (int i = 0; i < np; ++i) {
            double* o = out + MPFO_PLANE * i;
            o[6] = A[3 * i];
            o[7] = A[3 * i + 1];
            o[8] = A[3 * i + 2];
        }
        free(A);
    }
    free(dist);
}

/* ---------------------------------------------------------------------- */
/* batch drivers                                                           */
/* ---------------------------------------------------------------------- */
typedef struct {
    const mpfo_tree* T;
    const mpfo_cosmo* C;
    int order, stop_kind, nplanes, jac;
    double length, stop_ref;
    unsigned nsteps;
    const double* ki;
    const double* launch;
    const double* planes;
    int64_t* steps;
    double* final_out;
    double* plane_out;
    int64_t n;
    int64_t next;
    pthread_mutex_t mu;
} job_t;

static int64_t take(job_t* J)
{
    pthread_mutex_lock(&J->mu);
    const int64_t i = J->next++;
    pthread_mutex_unlock(&J->mu);
    return i;
}

static void* worker(void* arg)
{
    job_t* J = (job_t*)arg;
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    traj_t tr = {0, 0, 0};
    for (int64_t i; (i = take(J)) < J->n;) {
        c->T = J->T;
        c->C = J->C;
        c->order = J->order;
        c->length = J->length;
        cache_init(&c->cache);
        tr.n = 0;
        launch6(J->launch + 6 * i, traj_push(&tr));
        const double ref = (J->nplanes > 0) ? J->planes[J->nplanes - 1] : J->stop_ref;
        integrate(c, &tr, J->nsteps, J->stop_kind, ref, J->ki);
        J->steps[i] = tr.n;
        if (J->final_out) {
            if (tr.n > 0) memcpy(J->final_out + MPFO_PHOTON * i, tr.p + MPFO_PHOTON * (tr.n - 1), MPFO_PHOTON * sizeof(double));
            else memset(J->final_out + MPFO_PHOTON * i, 0, MPFO_PHOTON * sizeof(double));
        }
        if (J->nplanes > 0 && J->plane_out)
            planes_of(c, &tr, J->stop_kind, J->nplanes, J->planes, J->jac, J->plane_out + (int64_t)MPFO_PLANE * J->nplanes * i);
    }
    free(tr.p);
    free(c);
    return 0;
}

int mpfo_propagate(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                   int stop_kind, double stop_ref, const double* ki_target,
                   int64_t n, const double* launch, int nplanes, const double* planes, int jacobian_on,
                   int64_t* steps, double* final_out, double* plane_out, int nthreads)
{
    if (!T || !C || (order < 0 || order > 2) || nsteps == 0 || n < 0) return -1;
    static const double zero3[3] = {0, 0, 0};
    job_t J;
    J.T = T; J.C = C; J.order = order; J.stop_kind = stop_kind; J.nplanes = nplanes; J.jac = jacobian_on;
    J.length = length; J.stop_ref = stop_ref; J.nsteps = nsteps; J.ki = ki_target ? ki_target : zero3;
    J.launch = launch; J.planes = planes; J.steps = steps; J.final_out = final_out; J.plane_out = plane_out;
    J.n = n; J.next = 0;
    pthread_mutex_init(&J.mu, 0);
    if (nthreads <= 1) worker(&J);
    else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], 0, worker, &J);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], 0);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    return 0;
}

int64_t mpfo_trajectory(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                        int stop_kind, double stop_ref, const double* launch, double* out, int64_t cap)
{
    static const double zero3[3] = {0, 0, 0};
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    c->T = T; c->C = C; c->order = order; c->length = length;
    cache_init(&c->cache);
    traj_t tr = {0, 0, 0};
    launch6(launch, traj_push(&tr));
    integrate(c, &tr, nsteps, stop_kind, stop_ref, zero3);
    const int64_t m = tr.n;
    for (int64_t k = 0; k < m && k < cap; ++k) memcpy(out + MPFO_PHOTON * k, tr.p + MPFO_PHOTON * k, MPFO_PHOTON * sizeof(double));
    free(tr.p);
    free(c);
    return m;
}

/* ---------------------------------------------------------------------- */
/* ray bundles: Integrator::propagate (integrator.h:861-1015)              */
/* ---------------------------------------------------------------------- */
/* reference parameter of point k (integrator.h:925-969) */
static double bundle_ref(const double* tr, int64_t k, int kind)
{
    const double* p = tr + MPFO_PHOTON * k;
    switch (kind) {
    case MPFO_STOP_A: return 1 / p[PA] - 1;
    case MPFO_STOP_T: return p[PT];
    case MPFO_STOP_LAMBDA: return p[PLAMBDA];
    case MPFO_STOP_R: {
        const double dx = p[PX] - tr[PX], dy = p[PY] - tr[PY], dz = p[PZ] - tr[PZ];
        return sqrt(dx * dx + dy * dy + dz * dz);
    }
    default: return p[PZRED];
    }
}

/* Utility::interpolate (utility.h:441-449) of coordinate q of a ray at x0 */
static double bundle_interp(double x0, const double* tr, int64_t n, int kind, int q)
{
    int64_t first = 0, count = n;
    while (count > 0) {
        const int64_t step = count >> 1, it = first + step;
        if (!(x0 < bundle_ref(tr, it, kind))) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    int64_t i = first;
    i += (n > 1) * ((i <= 0) - (i >= n));
    if (n > 1) {
        const double xm = bundle_ref(tr, i - 1, kind), xi = bundle_ref(tr, i, kind);
        const double ym = tr[MPFO_PHOTON * (i - 1) + q], yi = tr[MPFO_PHOTON * i + q];
        return ym + ((yi - ym) * (x0 - xm) / (xi - xm));
    }
    return (n > 0) ? tr[q] : 0.0;
}

int64_t mpfo_propagate_bundle(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                              const double* photon, unsigned count, double angle, double rotation, int kind, double amin,
                              double* out, int64_t cap)
{
    static const double zero3[3] = {0, 0, 0};
    const unsigned total = count + 1;
    /* Integrator::launch(photon, count, angle, rotation), centre first (integrator.h:346-380) */
    double* dirs = (double*)malloc(sizeof(double) * 3 * total);
    {
        const double zero = 0, one = 1, four = 4;
        const double pi = four * atan(one);
        const double step = (pi + pi) / (double)(count + (!count));
        const double* k = photon + 3;
        const double r = sqrt((k[0] * k[0]) + (k[1] * k[1]) + (k[2] * k[2]));
        const double rcos = r * cos(angle), rsin = r * sin(angle);
        const double costheta = cos(acos(k[2] / r)), sintheta = sin(acos(k[2] / r));
        const double cosphi = cos(atan2(k[1], k[0])), sinphi = sin(atan2(k[1], k[0]));
        const double cospsi = cos(rotation), sinpsi = sin(rotation);
        for (unsigned q = 0; q < total; ++q)
            for (int d = 0; d < 3; ++d) dirs[3 * q + d] = k[d];
        if (r > zero) {
            for (unsigned istep = 0; istep < count; ++istep) {
                const double x = rsin * cos(istep * step), y = rsin * sin(istep * step), z = rcos;
                double* o = dirs + 3 * (istep + 1);
                o[0] = -cosphi * sinpsi * costheta * x - cosphi * cospsi * costheta * y + cosphi * sintheta * z + sinphi * sinpsi * y -
                       sinphi * cospsi * x;
                o[1] = -sinphi * sinpsi * costheta * x - sinphi * cospsi * costheta * y - cosphi * sinpsi * y + cosphi * cospsi * x +
                       sintheta * sinphi * z;
                o[2] = sintheta * sinpsi * x + sintheta * cospsi * y + costheta * z;
            }
        }
    }
    /* each ray integrated without a stop criterion (integrator.h:477-618) */
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    c->T = T; c->C = C; c->order = order; c->length = length;
    traj_t* trs = (traj_t*)calloc(total, sizeof(traj_t));
    double* last = (double*)calloc(total, sizeof(double));
    const double quarter = (4.0 / (2.0 * 1.0)) / 2.0, limit = 1.0 / (2.0 * 2.0 * 2.0);
    unsigned nt = total;
    for (unsigned it = 0; it < nt; ++it) {
        cache_init(&c->cache);
        double* p = traj_push(&trs[it]);
        launch6(photon, p);   /* a t x y z, then the given direction as is */
        p[PK1] = dirs[3 * it]; p[PK2] = dirs[3 * it + 1]; p[PK3] = dirs[3 * it + 2];
        integrate(c, &trs[it], nsteps, MPFO_STOP_R, INFINITY, zero3);
        const int64_t size = trs[it].n;
        if (!size) {
            nt = 0;
        } else {
            const double* front = trs[it].p;
            const double* back = trs[it].p + MPFO_PHOTON * (size - 1);
            const double cx = back[PX] - front[PX], cy = back[PY] - front[PY], cz = back[PZ] - front[PZ];
            last[it] = sqrt(cx * cx + cy * cy + cz * cz);
            nt *= (last[it] > quarter);
            nt *= (!(isnormal(amin) && isnormal(back[PAH]) && (back[PAH] < 1.0))) || (!(back[PAH] > amin));
        }
    }
    double mx = last[0], mn = last[0];
    for (unsigned it = 1; it < total; ++it) {
        if (last[it] > mx) mx = last[it];
        if (last[it] < mn) mn = last[it];
    }
    nt *= (fabs(mx - mn) / mx < limit);
    int64_t m = 0;
    if (nt > 0) {
        const double* T0 = trs[0].p;
        m = trs[0].n;
        for (int64_t k = 0; k < m && k < cap; ++k) {
            const double* p = T0 + MPFO_PHOTON * k;
            double d = 0.0;
            if (nt > 1) {
                const double x0 = bundle_ref(T0, k, kind);
                for (unsigned it = 1; it < nt; ++it) {
                    const double cx = bundle_interp(x0, trs[it].p, trs[it].n, kind, PX) - p[PX];
                    const double cy = bundle_interp(x0, trs[it].p, trs[it].n, kind, PY) - p[PY];
                    const double cz = bundle_interp(x0, trs[it].p, trs[it].n, kind, PZ) - p[PZ];
                    d += sqrt(cx * cx + cy * cy + cz * cz);
                }
                d /= (double)(nt - 1);
                d *= (length * p[PA]) / angle;
            }
            double* o = out + 29 * k;
            o[0] = p[PINDEX];
            for (int q = 0; q < 9; ++q) o[1 + q] = p[q];
            o[10] = p[PLEVEL]; o[11] = p[PAH]; o[12] = p[PRHO]; o[13] = p[PPHI];
            o[14] = p[PDX]; o[15] = p[PDY]; o[16] = p[PDZ]; o[17] = p[PDL]; o[18] = p[PLAP];
            o[19] = p[PZRED]; o[20] = p[PDS2]; o[21] = p[PERR]; o[22] = d;
            o[23] = p[PISW]; o[24] = p[PISWOLD]; o[25] = p[PCHI]; o[26] = p[PLAMBDA]; o[27] = p[PDT]; o[28] = p[PS];
        }
    }
    for (unsigned it = 0; it < total; ++it) free(trs[it].p);
    free(trs);
    free(last);
    free(dirs);
    free(c);
    return m;
}

/* ---------------------------------------------------------------------- */
/* catalogue root-finder                                                   */
/* ---------------------------------------------------------------------- */
/* Integrator::launch, (phi, theta) form (integrator.h:305-329). */
static void launch5(double phi, double theta, double* p)
{
    memset(p, 0, MPFO_PHOTON * sizeof(double));
    p[PA] = 1.0;
    p[PK0] = 1.0;
    p[PK1] = cos(phi) * sin(theta);
    p[PK2] = sin(phi) * sin(theta);
    p[PK3] = cos(theta);
}

typedef struct {
    const mpfo_tree* T;
    const mpfo_cosmo* C;
    int order, max_iterations;
    int bundle, plane_sachs, stop_bundle;   /* jacobiantype = bundle, plane = sachs, stop_bundle kind */
    double length, accuracy, h, mpc, openingmin;
    unsigned nsteps;
    const double* src;
    const double* rot;
    const double* vobs;
    double* out;
    int64_t n, next;
    pthread_mutex_t mu;
} cjob_t;

static void dbetadtheta(ctx_t* c, traj_t* tr, unsigned nsteps, int stop_bundle, double openingmin, int np,
                        const double* ki, const double* iref_v, const double* dist, double phiInit,
                        double thetaInit, double* J);

/* One Catalogues::newtonMethod2d call (catalogues.h:410-727) with
 * jacobiantype = infinitesimal and use_previous_catalogues = 0: res =
 * {{phi', theta'}, {miss, firstid}}; jac and z are updated in place as the
 * reference updates its jacobian and redshifts arguments. */
static void newton2d(ctx_t* c, traj_t* tr, traj_t* trb, const cjob_t* J, const double* target, const double* vel,
                     double dist, double phi, double theta, unsigned iteration, double res[2][2], double jac[2][2],
                     double* z)
{
    static const double cl = C_LIGHT, c2 = C_LIGHT * C_LIGHT;
    tr->n = 0;
    launch5(phi, theta, traj_push(tr));
    integrate(c, tr, J->nsteps, MPFO_STOP_R, dist, (const double[3]){0, 0, 0});
    const int64_t marked = tr->n - 1;
    const int64_t firstid = marked - (marked > 0);
    const double* P0 = tr->p + MPFO_PHOTON * firstid;
    if (marked == 0 || tr->p[MPFO_PHOTON * marked + PCHI] < dist) {
        res[0][0] = 42; res[0][1] = 42; res[1][0] = 0; res[1][1] = (double)firstid;
        return;
    }
    const double* P1 = P0 + MPFO_PHOTON;
    const double previous = P0[PCHI], next = P1[PCHI];
    const double f = (next - dist) / (next - previous);
    z[1] = P0[PZRED] * f + P1[PZRED] * (1 - f);
    const double scale_factor = P0[PA] * f + P1[PA] * (1 - f);
    double fp[3];
    fp[0] = P0[PX] * f + P1[PX] * (1 - f);
    fp[1] = P0[PY] * f + P1[PY] * (1 - f);
    fp[2] = P0[PZ] * f + P1[PZ] * (1 - f);
    /* jacobiantype = bundle: the screen normal and the bundle's stop value (catalogues.h:458-495) */
    double kiT[3] = {0, 0, 0}, iref = 0;
    if (J->bundle == 1) {
        if (J->plane_sachs) {
            kiT[0] = P0[PK1] * f + P1[PK1] * (1 - f);
            kiT[1] = P0[PK2] * f + P1[PK2] * (1 - f);
            kiT[2] = P0[PK3] * f + P1[PK3] * (1 - f);
        } else {
            kiT[0] = fp[0]; kiT[1] = fp[1]; kiT[2] = fp[2];
        }
        switch (J->stop_bundle) {
        case MPFO_STOP_REDSHIFT: iref = z[1]; break;
        case MPFO_STOP_A: iref = scale_factor; break;
        case MPFO_STOP_T: iref = P0[PT] * f + P1[PT] * (1 - f); break;
        case MPFO_STOP_LAMBDA: iref = P0[PLAMBDA] * f + P1[PLAMBDA] * (1 - f); break;
        case MPFO_STOP_R: iref = dist; break;
        default: iref = kiT[0] * fp[0] + kiT[1] * fp[1] + kiT[2] * fp[2]; break;
        }
    }
    const double dist_sep = sqrt(pow(target[0] - fp[0], 2) + pow(target[1] - fp[1], 2) + pow(target[2] - fp[2], 2));
    res[1][0] = dist_sep / dist;
    if (res[1][0] > J->accuracy) {
        double ji[2][2] = {{1, 0}, {0, 1}};
        if (iteration >= 5 && J->bundle == 1) {
            double B[4];
            dbetadtheta(c, trb, J->nsteps, J->stop_bundle, J->openingmin, 1, kiT, &iref, &dist, phi, theta, B);
            if (B[0] == 42 && B[1] == 42) {
                /* catalogues.h:521-528; the reference leaves result[1][1] unset here */
                res[0][0] = 42; res[0][1] = 42; res[1][0] = 22; res[1][1] = 0;
                return;
            }
            jac[0][0] = B[0]; jac[0][1] = B[1]; jac[1][0] = B[2]; jac[1][1] = B[3];
            const double invdet = 1. / (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]);
            ji[0][0] = jac[1][1] * invdet;
            ji[0][1] = -jac[0][1] * invdet;
            ji[1][0] = -jac[1][0] * invdet;
            ji[1][1] = jac[0][0] * invdet;
        } else if (iteration >= 3) {
            double A[3];
            jacobian(c, tr, 1, &dist, A);
            jac[0][0] = A[0]; jac[0][1] = A[1]; jac[1][0] = A[1]; jac[1][1] = A[2];
            /* Utility::invMatrix2d (utility.h:686-696) */
            const double invdet = 1. / (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]);
            ji[0][0] = jac[1][1] * invdet;
            ji[0][1] = -jac[0][1] * invdet;
            ji[1][0] = -jac[1][0] * invdet;
            ji[1][1] = jac[0][0] * invdet;
        }
        /* Newton step in the screen basis (catalogues.h:625-655) */
        const double cp = cos(phi), sp = sin(phi), ct = cos(theta), st = sin(theta);
        double e1[3], e2[3], sep[3], pos[3], targeted[3];
        e1[0] = -sp; e1[1] = cp; e1[2] = 0;
        e2[0] = -cp * ct; e2[1] = -sp * ct; e2[2] = st;
        targeted[0] = dist * cp * st;
        targeted[1] = dist * sp * st;
        targeted[2] = dist * ct;
        for (int k = 0; k < 3; ++k) {
            sep[k] = fp[k] - target[k];
            pos[k] = targeted[k] - target[k];
        }
        const double sepx = sep[0] * e1[0] + sep[1] * e1[1];
        const double sepy = sep[0] * e2[0] + sep[1] * e2[1] + sep[2] * e2[2];
        const double posx = pos[0] * e1[0] + pos[1] * e1[1];
        const double posy = pos[0] * e2[0] + pos[1] * e2[1] + pos[2] * e2[2];
        const double sepxnew = ji[0][0] * sepx + ji[0][1] * sepy;
        const double sepynew = ji[1][0] * sepx + ji[1][1] * sepy;
        const double posxnew = posx - sepxnew;
        const double posynew = posy - sepynew;
        const double xnew = target[0] + (posxnew * e1[0] + posynew * e2[0]);
        const double ynew = target[1] + (posxnew * e1[1] + posynew * e2[1]);
        const double znew = target[2] + posynew * e2[2];
        res[0][0] = atan2(ynew, xnew);
        res[0][1] = acos(znew / sqrt(xnew * xnew + ynew * ynew + znew * znew));
        return;
    }
    /* converged: Jacobian and redshift decomposition (catalogues.h:660-723) */
    if (J->bundle == 2) {
        /* infinitesimal_born (catalogues.h:670-673): the Order = -1 ray of the
           same launch to the source radius, the Jacobian along it */
        ctx_t cb = *c;
        cb.homogeneous = 1;
        trb->n = 0;
        launch5(phi, theta, traj_push(trb));
        integrate(&cb, trb, J->nsteps, MPFO_STOP_R, dist, (const double[3]){0, 0, 0});
        double A[3];
        jacobian(&cb, trb, 1, &dist, A);
        jac[0][0] = A[0]; jac[0][1] = A[1]; jac[1][0] = A[1]; jac[1][1] = A[2];
    } else if (J->bundle) {
        double B[4];
        dbetadtheta(c, trb, J->nsteps, J->stop_bundle, J->openingmin, 1, kiT, &iref, &dist, phi, theta, B);
        jac[0][0] = B[0]; jac[0][1] = B[1]; jac[1][0] = B[2]; jac[1][1] = B[3];
        if (B[0] == 42 && B[1] == 42) {
            res[0][0] = 42; res[0][1] = 42; res[1][0] = 22; res[1][1] = 0;
            return;
        }
    } else {
        double A[3];
        jacobian(c, tr, 1, &dist, A);
        jac[0][0] = A[0]; jac[0][1] = A[1]; jac[1][0] = A[1]; jac[1][1] = A[2];
    }
    const double* T0 = tr->p;
    const double* vo = J->vobs;
    const double potential = P0[PPHI] * f + P1[PPHI] * (1 - f);
    const double isw = P0[PISW] * f + P1[PISW] * (1 - f);
    z[0] = -1 + 1. / (scale_factor);
    const double unit_t = scale_factor * scale_factor * J->mpc / (J->h * 100.0 * 1000.0);
    const double unit_l = scale_factor * c->length * 100;
    const double velocityx = vel[0] * unit_l * 1e-2 / (unit_t * cl);
    const double velocityy = vel[1] * unit_l * 1e-2 / (unit_t * cl);
    const double velocityz = vel[2] * unit_l * 1e-2 / (unit_t * cl);
    const double gref = -T0[PA] * cl * T0[PK0] * (1. + T0[PPHI] / c2 + (vo[0] * T0[PK1] + vo[1] * T0[PK2] + vo[2] * T0[PK3]) / (cl * T0[PK0]) +
                                                   0.5 * (vo[0] * vo[0] + vo[1] * vo[1] + vo[2] * vo[2]));
    const double dtdl = P0[PK0] * f + P1[PK0] * (1 - f);
    const double dxdl = P0[PK1] * f + P1[PK1] * (1 - f);
    const double dydl = P0[PK2] * f + P1[PK2] * (1 - f);
    const double dzdl = P0[PK3] * f + P1[PK3] * (1 - f);
    const double gK = -scale_factor * cl * dtdl * (1. + potential / c2 + (velocityx * dxdl + velocityy * dydl + velocityz * dzdl) / (cl * dtdl) +
                                                    0.5 * (velocityx * velocityx + velocityy * velocityy + velocityz * velocityz));
    z[2] = z[1] + (velocityx * dxdl + velocityy * dydl + velocityz * dzdl) / (scale_factor * cl * dtdl) -
           (vo[0] * T0[PK1] + vo[1] * T0[PK2] + vo[2] * T0[PK3]) / (scale_factor * cl * T0[PK0]);
    z[3] = z[2] + 0.5 * (velocityx * velocityx + velocityy * velocityy + velocityz * velocityz - vo[0] * vo[0] - vo[1] * vo[1] - vo[2] * vo[2]) / scale_factor;
    z[4] = z[3] + isw / scale_factor;
    z[5] = gK / gref - 1;
    res[0][0] = phi;
    res[0][1] = theta;
}

/* FillMap's lensing_born rays (hmaps.h:706-712): per launch (6-argument
 * form), the Order = -1 ray (homogeneous field, the octree's levels for the
 * steps) to stop_ref of stop_kind, then Lensing::dbetadtheta_infinitesimal
 * along it at the nd distances (the FLRW surface distances).  size: the
 * Born trajectory sizes; A: n x nd x 3 (a11 a12 a22). */
int mpfo_born(const mpfo_tree* T, const mpfo_cosmo* C, double length, unsigned nsteps, int stop_kind, double stop_ref,
              int64_t n, const double* launch, int nd, const double* dist, int64_t* size, double* A)
{
    if (!T || !C || nsteps == 0 || n < 0 || nd < 1 || !launch || !dist || !size || !A) return -1;
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    traj_t tr = {0, 0, 0};
    const double zero3[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        c->T = T;
        c->C = C;
        c->order = 2;
        c->length = length;
        c->homogeneous = 1;
        cache_init(&c->cache);
        tr.n = 0;
        launch6(launch + 6 * i, traj_push(&tr));
        integrate(c, &tr, nsteps, stop_kind, stop_ref, zero3);
        size[i] = tr.n;
        jacobian(c, &tr, nd, dist, A + (int64_t)3 * nd * i);
    }
    free(tr.p);
    free(c);
    return 0;
}

/* Catalogues::iterateNewtonMethod (catalogues.h:757-783) behind relCat's
 * per-source setup and row (catalogues.h:811-856). */
static void catalogue_one(ctx_t* c, traj_t* tr, traj_t* trb, const cjob_t* J, int64_t i)
{
    const double* s = J->src + 6 * i;
    double target[3], vel[3];
    for (int j = 0; j < 3; ++j) {
        if (!J->rot) {
            target[j] = s[j];
            vel[j] = s[j + 3];
        } else {
            target[j] = s[0] * J->rot[3 * j + 0] + s[1] * J->rot[3 * j + 1] + s[2] * J->rot[3 * j + 2];
            vel[j] = s[3] * J->rot[3 * j + 0] + s[4] * J->rot[3 * j + 1] + s[5] * J->rot[3 * j + 2];
        }
    }
    const double dist = sqrt(target[0] * target[0] + target[1] * target[1] + target[2] * target[2]);
    const double theta = acos(target[2] / dist);
    const double phi = atan2(target[1], target[0]);
    double res[2][2] = {{phi, theta}, {0, 0}};
    double jac[2][2] = {{0, 0}, {0, 0}};
    double z[6] = {0, 0, 0, 0, 0, 0};
    unsigned iteration = 0;
    for (;;) {
        const double p0 = res[0][0], t0 = res[0][1];
        newton2d(c, tr, trb, J, target, vel, dist, p0, t0, iteration, res, jac, z);
        iteration++;
        if (res[0][0] == 42 && res[0][1] == 42) break;
        if (iteration > (unsigned)J->max_iterations && res[1][0] > J->accuracy) {
            res[1][1] = 42;
            break;
        }
        if (!(res[1][0] > J->accuracy)) {
            res[1][1] = iteration;
            break;
        }
    }
    double* o = J->out + 16 * i;
    o[0] = phi; o[1] = theta;
    o[2] = res[0][0]; o[3] = res[0][1]; o[4] = res[1][0]; o[5] = res[1][1];
    for (int k = 0; k < 6; ++k) o[6 + k] = z[k];
    o[12] = jac[0][0]; o[13] = jac[0][1]; o[14] = jac[1][0]; o[15] = jac[1][1];
}

static void* cworker(void* arg)
{
    cjob_t* J = (cjob_t*)arg;
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    traj_t tr = {0, 0, 0}, trb = {0, 0, 0};
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int64_t i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->n) break;
        c->T = J->T;
        c->C = J->C;
        c->order = J->order;
        c->length = J->length;
        cache_init(&c->cache);
        catalogue_one(c, &tr, &trb, J, i);
    }
    free(tr.p);
    free(trb.p);
    free(c);
    return 0;
}

int mpfo_catalogue(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                   int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                   double h, double mpc, int max_iterations, double* out, int nthreads)
{
    return mpfo_catalogue_jac(T, C, order, length, nsteps, n, src, rotm1, vobs, cat_accuracy, h, mpc, max_iterations,
                              0, 0, 0, 0.0, out, nthreads);
}

int mpfo_catalogue_jac(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                       int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                       double h, double mpc, int max_iterations, int bundle, int plane_sachs, int stop_bundle,
                       double openingmin, double* out, int nthreads)
{
    if (!T || !C || (order < 0 || order > 2) || nsteps == 0 || n < 0 || !vobs) return -1;
    cjob_t J;
    J.bundle = bundle; J.plane_sachs = plane_sachs; J.stop_bundle = stop_bundle; J.openingmin = openingmin;
    J.T = T; J.C = C; J.order = order; J.max_iterations = max_iterations; J.length = length;
    J.accuracy = cat_accuracy; J.h = h; J.mpc = mpc; J.nsteps = nsteps; J.src = src; J.rot = rotm1;
    J.vobs = vobs; J.out = out; J.n = n; J.next = 0;
    pthread_mutex_init(&J.mu, 0);
    if (nthreads <= 1) cworker(&J);
    else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], 0, cworker, &J);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], 0);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    return 0;
}

/* ---------------------------------------------------------------------- */
/* bundle Jacobian                                                         */
/* ---------------------------------------------------------------------- */
static double plane_dot(const double* p, const double* ki) { return p[PX] * ki[0] + p[PY] * ki[1] + p[PZ] * ki[2]; }

/* Lensing::dbetadtheta (lensing.h:148-336) for one central direction: four
 * rays on a screen at +-tan(openingmin), integrated with the stop_bundle
 * criterion to the last surface value, their crossings of every surface and
 * the finite-difference Jacobian projected on the screen of kiTargets[iref].
 * J: np x 4 (a11 a12 a21 a22), value-initialised to 0 as the reference's. */
static void dbetadtheta(ctx_t* c, traj_t* tr, unsigned nsteps, int stop_bundle, double openingmin, int np,
                        const double* ki /* np x 3 */, const double* iref_v, const double* dist, double phiInit,
                        double thetaInit, double* J)
{
    for (int i = 0; i < 4 * np; ++i) J[i] = 0.0;
    double* fp = (double*)calloc((size_t)np * 12, sizeof(double));   /* [iref][ray][3] */
    const double cp = cos(phiInit), sp = sin(phiInit), ct = cos(thetaInit), st = sin(thetaInit);
    double target[3], e1[3], e2[3], rini[4][3];
    target[0] = cp * st; target[1] = sp * st; target[2] = ct;
    e1[0] = -sp; e1[1] = cp; e1[2] = 0;
    e2[0] = -cp * ct; e2[1] = -sp * ct; e2[2] = st;
    const double to = tan(openingmin);
    rini[0][0] = target[0] + to * e1[0]; rini[0][1] = target[1] + to * e1[1]; rini[0][2] = target[2];
    rini[1][0] = target[0] - to * e1[0]; rini[1][1] = target[1] - to * e1[1]; rini[1][2] = target[2];
    rini[2][0] = target[0] - to * e2[0]; rini[2][1] = target[1] - to * e2[1]; rini[2][2] = target[2] - to * e2[2];
    rini[3][0] = target[0] + to * e2[0]; rini[3][1] = target[1] + to * e2[1]; rini[3][2] = target[2] + to * e2[2];
    const int q = stop_quantity(stop_bundle);
    for (int r = 0; r < 4; ++r) {
        const double L[6] = {0, 0, 0, rini[r][0], rini[r][1], rini[r][2]};
        tr->n = 0;
        launch6(L, traj_push(tr));
        integrate(c, tr, nsteps, stop_bundle, iref_v[np - 1], ki + 3 * (np - 1));
        const double* back = tr->p + MPFO_PHOTON * (tr->n - 1);
        for (int i = 0; i < np; ++i) {
            int fail;
            if (stop_bundle == MPFO_STOP_A) fail = back[PA] > iref_v[i];
            else if (stop_bundle == MPFO_STOP_PLANE) fail = plane_dot(back, ki + 3 * i) < iref_v[i];
            else fail = back[q] < iref_v[i];
            if (fail) {
                if (stop_bundle == MPFO_STOP_A) {
                    J[4 * i + 0] = 42; J[4 * i + 1] = 42; J[4 * i + 2] = 1; J[4 * i + 3] = 3;
                } else {
                    for (int k = 0; k < np; ++k) { J[4 * k + 0] = 42; J[4 * k + 1] = 42; J[4 * k + 2] = 1; J[4 * k + 3] = 0; }
                }
                free(fp);
                return;
            }
            int64_t marked;
            double next, previous;
            if (stop_bundle == MPFO_STOP_PLANE) {
                int64_t first = 0, count = tr->n;   /* upper_bound with val < x . ki */
                while (count > 0) {
                    const int64_t step = count / 2, it = first + step;
                    if (!(iref_v[i] < plane_dot(tr->p + MPFO_PHOTON * it, ki + 3 * i))) { first = it + 1; count -= step + 1; }
                    else count = step;
                }
                marked = first;
            } else {
                marked = upper_by(tr, q, iref_v[i], stop_bundle == MPFO_STOP_A);
            }
            const int64_t fid = marked - (marked > 0);
            const double* P0 = tr->p + MPFO_PHOTON * fid;
            const double* P1 = P0 + MPFO_PHOTON;
            if (stop_bundle == MPFO_STOP_PLANE) {
                next = plane_dot(P1, ki + 3 * i);
                previous = plane_dot(P0, ki + 3 * i);
            } else {
                next = P1[q];
                previous = P0[q];
            }
            const double f = (next - iref_v[i]) / (next - previous);
            double* o = fp + 12 * i + 3 * r;
            o[0] = P0[PX] * f + P1[PX] * (1 - f);
            o[1] = P0[PY] * f + P1[PY] * (1 - f);
            o[2] = P0[PZ] * f + P1[PZ] * (1 - f);
        }
    }
    for (int i = 0; i < np; ++i) {
        const double* f0 = fp + 12 * i;
        double rh[3], rv[3];
        for (int d = 0; d < 3; ++d) {
            rh[d] = f0[0 + d] - f0[3 + d];
            rv[d] = f0[6 + d] - f0[9 + d];
        }
        const double kx = ki[3 * i], ky = ki[3 * i + 1], kz = ki[3 * i + 2];
        const double phik = atan2(ky, kx);
        const double thetak = acos(kz / sqrt(kx * kx + ky * ky + kz * kz));
        const double cpk = cos(phik), spk = sin(phik), ctk = cos(thetak), stk = sin(thetak);
        double a1[3], a2[3];
        a1[0] = -spk; a1[1] = cpk; a1[2] = 0;
        a2[0] = -cpk * ctk; a2[1] = -spk * ctk; a2[2] = stk;
        J[4 * i + 0] = (rh[0] * a1[0] + rh[1] * a1[1]) / (2 * dist[i] * to);
        J[4 * i + 1] = (rv[0] * a1[0] + rv[1] * a1[1]) / (2 * dist[i] * to);
        J[4 * i + 2] = (rh[0] * a2[0] + rh[1] * a2[1] + rh[2] * a2[2]) / (-2 * dist[i] * to);
        J[4 * i + 3] = (rv[0] * a2[0] + rv[1] * a2[1] + rv[2] * a2[2]) / (-2 * dist[i] * to);
    }
    free(fp);
}

typedef struct {
    const mpfo_tree* T;
    const mpfo_cosmo* C;
    int order, stop_kind, np, plane_sachs, stop_bundle;
    double length, openingmin;
    unsigned nsteps;
    const double* launch;
    const double* planes;
    double* plane_out;
    double* jac_out;
    int64_t n, next;
    pthread_mutex_t mu;
} bjob_t;

static void* bworker(void* arg)
{
    bjob_t* J = (bjob_t*)arg;
    ctx_t* c = (ctx_t*)calloc(1, sizeof(ctx_t));
    traj_t tr = {0, 0, 0}, trb = {0, 0, 0};
    const int np = J->np;
    double* ki = (double*)malloc(sizeof(double) * 3 * (size_t)np);
    double* iv = (double*)malloc(sizeof(double) * (size_t)np);
    double* dist = (double*)malloc(sizeof(double) * (size_t)np);
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int64_t i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->n) break;
        c->T = J->T; c->C = J->C; c->order = J->order; c->length = J->length;
        cache_init(&c->cache);
        const double* L = J->launch + 6 * i;
        tr.n = 0;
        launch6(L, traj_push(&tr));
        integrate(c, &tr, J->nsteps, J->stop_kind, J->planes[np - 1], (const double[3]){0, 0, 0});
        double* po = J->plane_out + (int64_t)MPFO_PLANE * np * i;
        planes_of(c, &tr, J->stop_kind, np, J->planes, 0, po);
        /* FillMap's targets for the bundle (hmaps.h:653-693) */
        for (int s = 0; s < np; ++s) {
            const double* o = po + MPFO_PLANE * s;
            const int64_t fid = (int64_t)o[0];
            const double f = o[1];
            const int ok = fid + 1 < tr.n;
            double* k = ki + 3 * s;
            if (J->plane_sachs && ok) {
                const double* P0 = tr.p + MPFO_PHOTON * fid;
                const double* P1 = P0 + MPFO_PHOTON;
                k[0] = P0[PK1] * f + P1[PK1] * (1 - f);
                k[1] = P0[PK2] * f + P1[PK2] * (1 - f);
                k[2] = P0[PK3] * f + P1[PK3] * (1 - f);
            } else {
                k[0] = o[2]; k[1] = o[3]; k[2] = o[4];
            }
            dist[s] = o[5];
            switch (J->stop_bundle) {
            case MPFO_STOP_LAMBDA: iv[s] = o[13]; break;
            case MPFO_STOP_R: iv[s] = o[12]; break;
            case MPFO_STOP_REDSHIFT: iv[s] = o[11]; break;
            case MPFO_STOP_A: iv[s] = o[10]; break;
            case MPFO_STOP_T: iv[s] = o[9]; break;
            default: iv[s] = k[0] * o[2] + k[1] * o[3] + k[2] * o[4]; break;
            }
        }
        const double phi = atan2(L[4], L[3]);
        const double theta = acos(L[5]);
        dbetadtheta(c, &trb, J->nsteps, J->stop_bundle, J->openingmin, np, ki, iv, dist, phi, theta,
                    J->jac_out + 4 * (int64_t)np * i);
    }
    free(ki); free(iv); free(dist);
    free(tr.p); free(trb.p);
    free(c);
    return 0;
}

int mpfo_bundle(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps, int stop_kind,
                int64_t n, const double* launch, int np, const double* planes, int plane_sachs, int stop_bundle,
                double openingmin, double* plane_out, double* jac_out, int nthreads)
{
    if (!T || !C || (order < 0 || order > 2) || nsteps == 0 || n < 0 || np < 1 || !planes) return -1;
    bjob_t J;
    J.T = T; J.C = C; J.order = order; J.stop_kind = stop_kind; J.np = np; J.plane_sachs = plane_sachs;
    J.stop_bundle = stop_bundle; J.length = length; J.openingmin = openingmin; J.nsteps = nsteps;
    J.launch = launch; J.planes = planes; J.plane_out = plane_out; J.jac_out = jac_out; J.n = n; J.next = 0;
    pthread_mutex_init(&J.mu, 0);
    if (nthreads <= 1) bworker(&J);
    else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], 0, bworker, &J);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], 0);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    return 0;
}

typedef struct {
    const mpfo_tree* T;
    int64_t n;
    const double* xyz;
    void* out;
    int kind;
    int nthreads, tid;
} gjob_t;

static void* gworker(void* arg)
{
    gjob_t* g = (gjob_t*)arg;
    for (int64_t i = g->tid; i < g->n; i += g->nthreads) {
        const double* p = g->xyz + 3 * i;
        if (g->kind == 0) ((int64_t*)g->out)[i] = mpfo_locate(g->T, p[0], p[1], p[2]);
        else if (g->kind == 1) mpfo_cic(g->T, p[0], p[1], p[2], (float*)g->out + 7 * i);
        else if (g->kind == 3) mpfo_ngp(g->T, p[0], p[1], p[2], (float*)g->out + 7 * i);
        else mpfo_tsc(g->T, p[0], p[1], p[2], (float*)g->out + 7 * i);
    }
    return 0;
}

static void gbatch(const mpfo_tree* T, int64_t n, const double* xyz, void* out, int kind, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    gjob_t* g = (gjob_t*)malloc(sizeof(gjob_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) {
        g[t].T = T; g[t].n = n; g[t].xyz = xyz; g[t].out = out; g[t].kind = kind; g[t].nthreads = nthreads; g[t].tid = t;
        pthread_create(&th[t], 0, gworker, &g[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], 0);
    free(th);
    free(g);
}

void mpfo_batch_locate(const mpfo_tree* T, int64_t n, const double* xyz, int64_t* out, int nthreads) { gbatch(T, n, xyz, out, 0, nthreads); }
void mpfo_batch_cic(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads) { gbatch(T, n, xyz, out, 1, nthreads); }
void mpfo_batch_tsc(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads) { gbatch(T, n, xyz, out, 2, nthreads); }
void mpfo_batch_ngp(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads) { gbatch(T, n, xyz, out, 3, nthreads); }

/* ---------------------------------------------------------------------- */
/* velocity field deposit (hmaps.h:439-550, hmaps.cpp:395-441)             */
/* ---------------------------------------------------------------------- */
/* The exact key's position in the sorted keys, or -1 (upper_bound, then
   the element before it compared for equality: hmaps.h:468-470). */
static inline int64_t find_exact(const mpfo_tree* T, u128 K)
{
    const int64_t m = upper(T, K);
    const int64_t j = m - (m > 0);
    return (T->n > 0 && tkey(T, j) == K) ? j : -1;
}

static inline double tsc_w(int a, double d);

int mpfo_velocity_deposit(const mpfo_tree* T, float* fields, float* v, int scheme, int64_t npart, const float* pos,
                          const float* pv, int flags)
{
    if (!T || T->n <= 0 || (scheme != 1 && scheme != 2)) return -1;
    unsigned lmin = 64, lmax = 0;
    for (int64_t i = 0; i < T->n; ++i) {
        const unsigned l = key_level(tkey(T, i));
        if (l < lmin) lmin = l;
        if (l > lmax) lmax = l;
    }
    if (flags & 1) {
        for (int64_t i = 0; i < T->n; ++i) {
            fields[7 * i] = 0.0f;
            v[3 * i] = v[3 * i + 1] = v[3 * i + 2] = 0.0f;
        }
    }
    for (unsigned L = lmin; L <= lmax; ++L) {
        const double half = 0.5 * OCT_EXTENT / pow(2, L);
        const double tw = 2 * half;
        const double invext = 1 / (OCT_EXTENT / pow(2, L));
        for (int64_t i = 0; i < npart; ++i) {
            const float* p = pos + 3 * i;
            if (scheme == 1) {
                for (int iz = -1; iz <= 1; iz += 2)
                    for (int iy = -1; iy <= 1; iy += 2)
                        for (int ix = -1; ix <= 1; ix += 2) {
                            const u128 K = key_compute(L, p[0] + half * ix, p[1] + half * iy, p[2] + half * iz);
                            const int64_t j = find_exact(T, K);
                            if (j < 0) continue;
                            const double w = (1 - fabs(p[0] - key_center(K, 0)) * invext) *
                                             (1 - fabs(p[1] - key_center(K, 1)) * invext) *
                                             (1 - fabs(p[2] - key_center(K, 2)) * invext);
                            fields[7 * j] += w;
                            for (int d = 0; d < 3; ++d) v[3 * j + d] += pv[3 * i + d] * w;
                        }
            } else {
                for (int iz = -1; iz <= 1; ++iz)
                    for (int iy = -1; iy <= 1; ++iy)
                        for (int ix = -1; ix <= 1; ++ix) {
                            const u128 K = key_compute(L, p[0] + tw * ix, p[1] + tw * iy, p[2] + tw * iz);
                            const int64_t j = find_exact(T, K);
                            if (j < 0) continue;
                            double dist[3];
                            for (int d = 0; d < 3; ++d) dist[d] = fabs((key_center(tkey(T, j), d) - p[d]) / tw);
                            const double w = tsc_w(abs(ix), dist[0]) * tsc_w(abs(iy), dist[1]) * tsc_w(abs(iz), dist[2]);
                            fields[7 * j] += w;
                            for (int d = 0; d < 3; ++d) v[3 * j + d] += pv[3 * i + d] * w;
                        }
            }
        }
    }
    if (flags & 2) {
        for (int64_t i = 0; i < T->n; ++i) {
            double mass = fields[7 * i];
            mass = mass + (mass == 0);
            for (int d = 0; d < 3; ++d) v[3 * i + d] /= mass;
        }
        for (unsigned L = lmin + 1; L <= lmax; ++L)
            for (int64_t i = 0; i < T->n; ++i) {
                const u128 k = tkey(T, i);
                if (key_level(k) != L || isnormal(fields[7 * i])) continue;
                const int64_t j = find_exact(T, key_parent(k));
                if (j < 0) continue;
                for (int d = 0; d < 3; ++d) v[3 * i + d] = v[3 * j + d];
            }
    }
    return 0;
}
