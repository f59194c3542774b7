// cz_arith.cuh -- bit-exact evaluation of the reference's wavelet stencils
// without binary64 arithmetic.
//
// The reference evaluates every stencil in binary64 and rounds to binary32 on
// return: `5./16 * f0 + 15./16 * f1 - 5./16 * f2 + 1./16 * f3` with float
// arguments and a float return type (WaveletsOnInterval.h:33-83). GB300 runs
// binary64 at a small fraction of its binary32 rate, so the kernels compute
// the same bits in binary32:
//
//   * A stencil is sum_i (k_i/D) * v_i with small integers k_i and D in
//     {8,16}. Every product is exact in binary64; whenever the exponents of
//     the inputs are within a bounded spread, every binary64 partial sum is
//     exact too, so the reference result is RN32(exact sum).
//   * Each input v is split against a line-wide grid U = 2^(E+1-B), E being
//     the exponent of the largest input of the line: v = hi + lo with
//     hi = RN_U(v) (two adds with the constant 1.5*2^(E+24-B)) and
//     lo = v - hi, both exact. The hi parts are integers times U of at most
//     2^B, so sum (k/D)*hi is exact in binary32 while K*2^B <= 2^24
//     (K = sum|k_i|). The lo parts are multiples of the smallest input ulp
//     and at most U/2, so sum (k/D)*lo is exact while
//     E - e_min <= B + 1 - log2(K). One final rounded add gives
//     RN32(exact sum). Grids and spreads per stencil are listed below.
//   * Lines whose spread is wider, or whose values sit near the ends of the
//     binary32 range, take the per-stencil path: the same split against the
//     stencil's own maximum, and binary64 only when even that is too wide.
//
// Signed zeros follow the binary64 chain: when the hi sum is zero the result
// is the lo chain itself, evaluated left to right like the reference.
//
// All binary32 arithmetic goes through explicit round-to-nearest intrinsics so
// the compiler cannot contract or reassociate it; host builds use
// -ffp-contract=off and the C99 fmaf.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CZ_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define CZ_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define CZ_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define CZ_ADD(a, b) __fadd_rn((a), (b))
#define CZ_SUB(a, b) __fsub_rn((a), (b))
#define CZ_MUL(a, b) __fmul_rn((a), (b))
#define CZ_DADD(a, b) __dadd_rn((a), (b))
#define CZ_DMUL(a, b) __dmul_rn((a), (b))
#define CZ_D2F(a) __double2float_rn(a)
#define CZ_BITS(x) __float_as_uint(x)
#define CZ_FLT(u) __uint_as_float(u)
#define CZ_UMIN(a, b) min((a), (b))
#define CZ_UMAX(a, b) max((a), (b))
#else
#define CZ_FMA(a, b, c) fmaf((a), (b), (c))
#define CZ_ADD(a, b) ((float)((a) + (b)))
#define CZ_SUB(a, b) ((float)((a) - (b)))
#define CZ_MUL(a, b) ((float)((a) * (b)))
#define CZ_DADD(a, b) ((double)(a) + (double)(b))
#define CZ_DMUL(a, b) ((double)(a) * (double)(b))
#define CZ_D2F(a) ((float)(a))
CZ_HD uint32_t cz_bits_h(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}
CZ_HD float cz_flt_h(uint32_t u)
{
    float x;
    memcpy(&x, &u, 4);
    return x;
}
#define CZ_BITS(x) cz_bits_h(x)
#define CZ_FLT(u) cz_flt_h(u)
#define CZ_UMIN(a, b) ((a) < (b) ? (a) : (b))
#define CZ_UMAX(a, b) ((a) > (b) ? (a) : (b))
#endif

namespace cz {

// Split grids and spreads. A line's sources are split against U = 2^(E+1-B)
// (E: exponent of the line maximum). Exactness needs, for a stencil with
// coefficient sum K = sum|k_i|:
//   hi sums:  K * 2^B <= 2^24
//   lo sums:  E - e_min <= B + 1 - log2(K)   (e_min: smallest non-zero input)
// B = 19 serves every stencil with K <= 32 with a spread of 15 binades
// (interp first/middle/one-to-last: K = 26/20/26; average-interpolating
// predictors: K <= 16). interp_last (K = 96) is re-split on B = 17, spread 11.
constexpr int kGridBits = 19;
constexpr int kSpread = 15;
constexpr int kLastGridBits = 17;
constexpr int kLastSpread = 11;

// Stencil coefficient sets k/D, exactly representable in binary32.
// WaveletsOnInterval.h:33-51 (D = 16) and :55-83 (D = 8).
struct W1F { static constexpr float c[4] = {5.f / 16, 15.f / 16, -5.f / 16, 1.f / 16}; };
struct W1M { static constexpr float c[4] = {-1.f / 16, 9.f / 16, 9.f / 16, -1.f / 16}; };
struct W1O { static constexpr float c[4] = {1.f / 16, -5.f / 16, 15.f / 16, 5.f / 16}; };
struct W1L { static constexpr float c[4] = {-5.f / 16, 21.f / 16, -35.f / 16, 35.f / 16}; };
struct P0F { static constexpr float c[3] = {11.f / 8, -1.f / 2, 1.f / 8}; };
struct P1F { static constexpr float c[3] = {5.f / 8, 1.f / 2, -1.f / 8}; };
struct P0M { static constexpr float c[3] = {1.f / 8, 1.f, -1.f / 8}; };
struct P1M { static constexpr float c[3] = {-1.f / 8, 1.f, 1.f / 8}; };
struct P0L { static constexpr float c[3] = {-1.f / 8, 1.f / 2, 5.f / 8}; };
struct P1L { static constexpr float c[3] = {1.f / 8, -1.f / 2, 11.f / 8}; };

// Exponent analysis of a set of stencil sources: biased exponent of the
// largest magnitude, and whether every non-zero source lies within `spread`
// binades of it (with the range limits that keep all grids representable:
// 27 <= eb keeps every grid at or above 2^-149, eb <= 247 keeps the split
// constants finite; an all-zero set is exact with any constant).
template <int H>
CZ_HD uint32_t max_bits(const float (&v)[H])
{
    uint32_t amax = 0;
#pragma unroll
    for (int i = 0; i < H; ++i) amax = CZ_UMAX(amax, CZ_BITS(v[i]) & 0x7fffffffu);
    return amax;
}
template <int H>
CZ_HD bool within(const float (&v)[H], uint32_t amax, int spread)
{
    const uint32_t eb = amax >> 23;
    // non-zero |v| below 2^(E-spread)  <=>  (bits-1) < (threshold bits - 1)
    const uint32_t tb = ((eb - (uint32_t)spread) << 23) - 1u;
    uint32_t small = 0;
#pragma unroll
    for (int i = 0; i < H; ++i) small |= (uint32_t)(((CZ_BITS(v[i]) & 0x7fffffffu) - 1u) < tb);
    return (amax == 0u) || (eb >= 27u && eb <= 247u && !small);
}

// Split constant 1.5*2^(E+24-B); its ulp is the grid U = 2^(E+1-B).
template <int B>
CZ_HD float split_const(uint32_t amax)
{
    const uint32_t eb = amax == 0u ? 127u : CZ_UMIN(CZ_UMAX(amax >> 23, 27u), 247u);
    return CZ_FLT(((eb + (uint32_t)(24 - B)) << 23) | 0x400000u);
}

template <int H>
CZ_HD void split(const float (&v)[H], float C, float (&hi)[H], float (&lo)[H])
{
#pragma unroll
    for (int i = 0; i < H; ++i) {
        hi[i] = CZ_SUB(CZ_ADD(v[i], C), C);
        lo[i] = CZ_SUB(v[i], hi[i]);
    }
}

// Line-level analysis and split on the main grid. Returns true when the
// binary32 fast path is exact for every stencil with K <= 32 on this line.
// One pass gives the largest magnitude and the smallest non-zero one (as
// bits - 1, unsigned, so that zeros never count); the spread test of
// `within` is then one compare.
template <int H>
CZ_HD bool line_split(const float (&v)[H], float (&hi)[H], float (&lo)[H], uint32_t &amax)
{
    uint32_t mx = 0, mn1 = 0xffffffffu;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        const uint32_t m = CZ_BITS(v[i]) & 0x7fffffffu;
        mx = CZ_UMAX(mx, m);
        mn1 = CZ_UMIN(mn1, m - 1u);
    }
    amax = mx;
    split<H>(v, split_const<kGridBits>(mx), hi, lo);
    const uint32_t eb = mx >> 23;
    const uint32_t tb = ((eb - (uint32_t)kSpread) << 23) - 1u;
    return (mx == 0u) || (eb >= 27u && eb <= 247u && mn1 >= tb);
}

// RN32 of sum c_i*(hi_i+lo_i) given an exact split (see header).
template <class S>
CZ_HD float st4_fast(float h0, float h1, float h2, float h3, float l0, float l1, float l2, float l3)
{
    float sh = CZ_MUL(S::c[0], h0);
    sh = CZ_FMA(S::c[1], h1, sh);
    sh = CZ_FMA(S::c[2], h2, sh);
    sh = CZ_FMA(S::c[3], h3, sh);
    float sl = CZ_MUL(S::c[0], l0);
    sl = CZ_FMA(S::c[1], l1, sl);
    sl = CZ_FMA(S::c[2], l2, sl);
    sl = CZ_FMA(S::c[3], l3, sl);
    return sh == 0.f ? sl : CZ_ADD(sh, sl);
}
template <class S>
CZ_HD float st3_fast(float h0, float h1, float h2, float l0, float l1, float l2)
{
    float sh = CZ_MUL(S::c[0], h0);
    sh = CZ_FMA(S::c[1], h1, sh);
    sh = CZ_FMA(S::c[2], h2, sh);
    float sl = CZ_MUL(S::c[0], l0);
    sl = CZ_FMA(S::c[1], l1, sl);
    sl = CZ_FMA(S::c[2], l2, sl);
    return sh == 0.f ? sl : CZ_ADD(sh, sl);
}

// The reference arithmetic itself: binary64 products summed left to right,
// rounded to binary32 once (used when no exact binary32 split exists).
template <class S>
CZ_HD float st4_f64(float v0, float v1, float v2, float v3)
{
    double s = CZ_DMUL((double)S::c[0], (double)v0);
    s = CZ_DADD(s, CZ_DMUL((double)S::c[1], (double)v1));
    s = CZ_DADD(s, CZ_DMUL((double)S::c[2], (double)v2));
    s = CZ_DADD(s, CZ_DMUL((double)S::c[3], (double)v3));
    return CZ_D2F(s);
}
template <class S>
CZ_HD float st3_f64(float v0, float v1, float v2)
{
    double s = CZ_DMUL((double)S::c[0], (double)v0);
    s = CZ_DADD(s, CZ_DMUL((double)S::c[1], (double)v1));
    s = CZ_DADD(s, CZ_DMUL((double)S::c[2], (double)v2));
    return CZ_D2F(s);
}

// Per-stencil path: split against the stencil's own maximum (grid chosen by
// the stencil's coefficient sum); binary64 when even that is too wide.
template <class S, int B, int SPREAD>
CZ_HD float st4_any(float v0, float v1, float v2, float v3)
{
    const float v[4] = {v0, v1, v2, v3};
    const uint32_t amax = max_bits<4>(v);
    if (within<4>(v, amax, SPREAD)) {
        float h[4], l[4];
        split<4>(v, split_const<B>(amax), h, l);
        return st4_fast<S>(h[0], h[1], h[2], h[3], l[0], l[1], l[2], l[3]);
    }
    return st4_f64<S>(v0, v1, v2, v3);
}
template <class S>
CZ_HD float st3_any(float v0, float v1, float v2)
{
    const float v[3] = {v0, v1, v2};
    const uint32_t amax = max_bits<3>(v);
    if (within<3>(v, amax, kSpread)) {
        float h[3], l[3];
        split<3>(v, split_const<kGridBits>(amax), h, l);
        return st3_fast<S>(h[0], h[1], h[2], l[0], l[1], l[2]);
    }
    return st3_f64<S>(v0, v1, v2);
}

template <class S>
CZ_HD float st4_main(float v0, float v1, float v2, float v3)
{
    return st4_any<S, kGridBits, kSpread>(v0, v1, v2, v3);
}
CZ_HD float st4_lastany(float v0, float v1, float v2, float v3)
{
    return st4_any<W1L, kLastGridBits, kLastSpread>(v0, v1, v2, v3);
}

// interp_last on the line's last four sources, given the line maximum: its
// own coarser split (K = 96), per-stencil path when the spread is too wide.
CZ_HD float interp_last(float v0, float v1, float v2, float v3, uint32_t line_amax)
{
    const float v[4] = {v0, v1, v2, v3};
    if (within<4>(v, line_amax, kLastSpread)) {
        float h[4], l[4];
        split<4>(v, split_const<kLastGridBits>(line_amax), h, l);
        return st4_fast<W1L>(h[0], h[1], h[2], h[3], l[0], l[1], l[2], l[3]);
    }
    return st4_lastany(v0, v1, v2, v3);
}

}  // namespace cz
