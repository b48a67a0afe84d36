/* 128-bit octree keys of the C oracle (SimpleHyperOctreeIndex<__uint128_t, 3>
 * with EXTENT = 4): level src/magrathea/simplehyperoctreeindex.h:572-575,
 * parent/child :679-694, center :888-893, extent :950-955, containing
 * :997-1001, compute/cipher :1165-1189.
 * TEST INFRASTRUCTURE ONLY, shared by mpf_oracle.c and mpf_oracle_cells.c. */
#ifndef MPF_ORACLE_KEYS_H
#define MPF_ORACLE_KEYS_H
#include <stdint.h>

typedef unsigned __int128 u128;

#define OCT_EXTENT 4
#define LEVEL_SHIFT 2  /* log2(EXTENT) */

static inline u128 mk(uint64_t hi, uint64_t lo) { return ((u128)hi << 64) | lo; }
static inline u128 markers(void) { return mk(0x8888888888888888ULL, 0x8888888888888888ULL); }
static inline u128 invalid_key(void) { return (((u128)1) << 127) - 1; }

static inline unsigned ctz128(u128 m)
{
    const uint64_t lo = (uint64_t)m;
    if (lo) return (unsigned)__builtin_ctzll(lo);
    const uint64_t hi = (uint64_t)(m >> 64);
    return hi ? 64u + (unsigned)__builtin_ctzll(hi) : 128u;
}

static inline unsigned key_level(u128 k)
{
    const u128 m = k & markers();
    const unsigned tz = m ? ctz128(m) : 128u;
    return (128u - tz) / 4u + (k != 0);
}

static inline int key_containing(u128 a, u128 b)
{
    const u128 x = a ^ b;
    return ((~markers() & x) <= (markers() & x)) && (a <= b);
}

static inline u128 key_parent(u128 k)
{
    const unsigned loc = 132u - key_level(k) * 4u;
    const u128 mask = (loc < 128u) ? (~(u128)0) << loc : (u128)0;
    return k & mask;
}

static inline u128 key_child(u128 k, unsigned site)
{
    const unsigned l = key_level(k);
    if (l >= 32u) return k;
    return k | ((u128)((site & 7u) | 8u) << (128u - (l + 1u) * 4u));
}

static inline uint64_t axis_coord(unsigned level, double x)
{
    const double scale = (1.0 / (double)OCT_EXTENT) * (double)(((u128)1) << level);
    const double v = scale * (x - (-(double)OCT_EXTENT / 2.0));
    uint64_t c;
    if (!(v > 0.0)) c = 0;                         /* reference: undefined for v < 0 */
    else if (v >= 18446744073709551616.0) c = ~0ULL;
    else c = (uint64_t)v;
    return (level >= 64) ? c : (c & ((1ULL << level) - 1ULL));
}

static inline u128 key_compute(unsigned level, double x, double y, double z)
{
    if (level == 0) return 0;
    const uint64_t cx = axis_coord(level, x), cy = axis_coord(level, y), cz = axis_coord(level, z);
    u128 k = 0;
    for (unsigned i = 1; i <= level; ++i) {
        const unsigned b = level - i;
        const unsigned nib = 8u | (unsigned)(((cz >> b) & 1u) << 2) | (unsigned)(((cy >> b) & 1u) << 1) | (unsigned)((cx >> b) & 1u);
        k |= (u128)nib << (128u - 4u * i);
    }
    return k;
}

static inline double key_center(u128 k, unsigned dim)
{
    const unsigned l = key_level(k);
    uint64_t c = 0;
    for (unsigned i = 0; i < 32u; ++i) c |= (uint64_t)((k >> (128u - 4u * (i + 1u) + dim)) & 1u) << (31u - i);
    c >>= (32u - l);
    return (-(double)OCT_EXTENT / 2.0) +
           ((double)OCT_EXTENT * ((double)(2 * (u128)c + 1) / (double)(((u128)1) << (l + 1u))));
}

/* extent() with the default unit extent: 1 / 2^level */
static inline double key_extent1(u128 k) { return 1.0 / (1.0 * (double)(((u128)1) << key_level(k))); }
/* extent<double, ratio<0>, ratio<EXTENT>>(): EXTENT / 2^level */
static inline double key_extent4(u128 k) { return (double)OCT_EXTENT / (1.0 * (double)(((u128)1) << key_level(k))); }

#endif
