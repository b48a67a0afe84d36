// 128-bit octree keys and cell geometry, host and device.
//
// Restates SimpleHyperOctreeIndex<__uint128_t, 3> with EXTENT = 4
// (src/magrathea/simplehyperoctreeindex.h): level :572-575, containing
// :997-1001, compute/cipher :1165-1189, center :888-893, extent :950-955.
// A key is kept as (hi, lo) 64-bit halves; level L uses the top 4L bits, one
// nibble 1zyx per level from the most significant end.
//
// The integer coordinate of position x at level L is
//     trunc((1/4 * 2^L) * (x - (-2)))      (float64, in that order)
// masked to L bits.  Every function that feeds a comparison with the
// reference is evaluated in IEEE float64 without contraction; the CUDA
// sources that include this header are compiled with -fmad=false.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define MPF_HD __host__ __device__ __forceinline__
#else
#define MPF_HD inline
#endif

namespace mpf {

constexpr int kExtent = 4;
constexpr int kLevelShift = 2;   // log2(kExtent)
constexpr int kMaxLevel = 32;

struct Key {
    uint64_t hi, lo;
};

// 2^e as a double, built from its exponent bits (|e| <= 1022): the cell
// sizes and scales below are powers of two, so they need neither an
// int-to-double conversion nor a division, and are exact.
MPF_HD double pow2(int e)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)(1023 + e) << 52);
#else
    return std::ldexp(1.0, e);
#endif
}

MPF_HD bool key_less(Key a, Key b) { return (a.hi < b.hi) || (a.hi == b.hi && a.lo < b.lo); }
MPF_HD bool key_le(Key a, Key b) { return !key_less(b, a); }
MPF_HD bool key_eq(Key a, Key b) { return a.hi == b.hi && a.lo == b.lo; }

// Integer coordinate along one axis at `level`; negative values saturate to 0
// (the reference's conversion is undefined there; valid rays never get there).
MPF_HD uint64_t axis_coord(int level, double x)
{
    const double scale = pow2(level - kLevelShift);   // (1 / EXTENT) * 2^level, exact
    const double v = scale * (x - (-(double)kExtent / 2.0));
    uint64_t c = (v > 0.0) ? (uint64_t)v : 0ull;
    return (level >= 64) ? c : (c & ((1ull << level) - 1ull));
}

// Key of the level-`level` cell with integer coordinates (cx, cy, cz).
MPF_HD Key key_from_coords(int level, uint64_t cx, uint64_t cy, uint64_t cz)
{
    Key k{0, 0};
    for (int i = 1; i <= level; ++i) {
        const int b = level - i;
        const uint64_t nib = 8ull | (((cz >> b) & 1ull) << 2) | (((cy >> b) & 1ull) << 1) | ((cx >> b) & 1ull);
        if (i <= 16) k.hi |= nib << (64 - 4 * i);
        else k.lo |= nib << (128 - 4 * i);
    }
    return k;
}

MPF_HD int key_level(Key k)
{
    // (128 - tzcnt(k & markers)) / 4 + (k != 0)
    const uint64_t M = 0x8888888888888888ull;
    const uint64_t mlo = k.lo & M, mhi = k.hi & M;
    int tz;
#if defined(__CUDA_ARCH__)
    if (mlo) tz = __ffsll((long long)mlo) - 1;
    else if (mhi) tz = 64 + __ffsll((long long)mhi) - 1;
    else tz = 128;
#else
    if (mlo) tz = __builtin_ctzll(mlo);
    else if (mhi) tz = 64 + __builtin_ctzll(mhi);
    else tz = 128;
#endif
    return (128 - tz) / 4 + ((k.hi | k.lo) != 0);
}

// Cell centre along one axis from its integer coordinate at `level`
// (exact in float64 for level <= 32).
MPF_HD double coord_center(int level, uint64_t c)
{
    // EXTENT * ((2c + 1) / 2^(L+1)) == (2c + 1) * 2^(2-L-1) exactly (powers of two)
    return (-(double)kExtent / 2.0) + (double)(2ull * c + 1ull) * pow2(kLevelShift - level - 1);
}

// Half of the cell size at `level`, in octree units, as the reference
// computes it: EXTENT/1 * (1/(1*2^L)) / 2.
MPF_HD double half_cell(int level)
{
    return pow2(kLevelShift - level - 1);   // EXTENT/1 * (1/2^L) / 2, exact
}

// extent<double, ratio<0>, ratio<EXTENT>>(): EXTENT / (1 * 2^L).
MPF_HD double cell_extent(int level) { return pow2(kLevelShift - level); }

}  // namespace mpf
