// cz_line.cuh -- one 1D interval-wavelet transform of a line held in
// registers, bit-exact to WI4::transform<N,forward> (WaveletsOnInterval.h:85-201).
//
// Layout of a transformed line: [N/2 scalings | N/2 details] along the line.
// wtype 1: 4th-order interpolating; 2: the same with the lifting update of the
// scalings; any other value: 3rd-order average-interpolating (the reference
// treats wtype 0 and 3 alike, :154).
#pragma once
#include "cz_arith.cuh"

namespace cz {

// ---------------------------------------------------------------- wtype 1/2
template <int N>
CZ_HD void fwd_interp(float (&x)[N], bool lifting)
{
    constexpr int H = N / 2;
    float e[H], h[H], l[H], d[H];
    uint32_t amax;
#pragma unroll
    for (int i = 0; i < H; ++i) e[i] = x[2 * i];
    if (line_split<H>(e, h, l, amax)) {
        d[0] = CZ_SUB(x[1], st4_fast<W1F>(h[0], h[1], h[2], h[3], l[0], l[1], l[2], l[3]));
#pragma unroll
        for (int i = 1; i < H - 2; ++i)
            d[i] = CZ_SUB(x[2 * i + 1], st4_fast<W1M>(h[i - 1], h[i], h[i + 1], h[i + 2], l[i - 1], l[i], l[i + 1],
                                                      l[i + 2]));
        d[H - 2] = CZ_SUB(x[N - 3], st4_fast<W1O>(h[H - 4], h[H - 3], h[H - 2], h[H - 1], l[H - 4], l[H - 3],
                                                  l[H - 2], l[H - 1]));
        d[H - 1] = CZ_SUB(x[N - 1], interp_last(e[H - 4], e[H - 3], e[H - 2], e[H - 1], amax));
    } else {
        d[0] = CZ_SUB(x[1], st4_main<W1F>(e[0], e[1], e[2], e[3]));
#pragma unroll
        for (int i = 1; i < H - 2; ++i)
            d[i] = CZ_SUB(x[2 * i + 1], st4_main<W1M>(e[i - 1], e[i], e[i + 1], e[i + 2]));
        d[H - 2] = CZ_SUB(x[N - 3], st4_main<W1O>(e[H - 4], e[H - 3], e[H - 2], e[H - 1]));
        d[H - 1] = CZ_SUB(x[N - 1], st4_lastany(e[H - 4], e[H - 3], e[H - 2], e[H - 1]));
    }
    // scalings[i] += 0.5*details[i] in binary64, rounded to binary32 (:124-126):
    // a single fma is the correctly rounded value of the same exact sum.
#pragma unroll
    for (int i = 0; i < H; ++i) x[i] = lifting ? CZ_FMA(0.5f, d[i], e[i]) : e[i];
#pragma unroll
    for (int i = 0; i < H; ++i) x[H + i] = d[i];
}

template <int N>
CZ_HD void inv_interp(float (&x)[N], bool lifting)
{
    constexpr int H = N / 2;
    float s[H], d[H], h[H], l[H], o[H];
    uint32_t amax;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        d[i] = x[H + i];
        s[i] = lifting ? CZ_FMA(-0.5f, d[i], x[i]) : x[i];  // :137-139
    }
    if (line_split<H>(s, h, l, amax)) {
        o[0] = st4_fast<W1F>(h[0], h[1], h[2], h[3], l[0], l[1], l[2], l[3]);
#pragma unroll
        for (int i = 1; i < H - 2; ++i)
            o[i] = st4_fast<W1M>(h[i - 1], h[i], h[i + 1], h[i + 2], l[i - 1], l[i], l[i + 1], l[i + 2]);
        o[H - 2] = st4_fast<W1O>(h[H - 4], h[H - 3], h[H - 2], h[H - 1], l[H - 4], l[H - 3], l[H - 2], l[H - 1]);
        o[H - 1] = interp_last(s[H - 4], s[H - 3], s[H - 2], s[H - 1], amax);
    } else {
        o[0] = st4_main<W1F>(s[0], s[1], s[2], s[3]);
#pragma unroll
        for (int i = 1; i < H - 2; ++i) o[i] = st4_main<W1M>(s[i - 1], s[i], s[i + 1], s[i + 2]);
        o[H - 2] = st4_main<W1O>(s[H - 4], s[H - 3], s[H - 2], s[H - 1]);
        o[H - 1] = st4_lastany(s[H - 4], s[H - 3], s[H - 2], s[H - 1]);
    }
    // :141-151: even samples are the scalings, odd samples interp + detail
#pragma unroll
    for (int i = 0; i < H; ++i) {
        x[2 * i] = s[i];
        x[2 * i + 1] = CZ_ADD(o[i], d[i]);
    }
}

// ---------------------------------------------------------------- wtype 3
template <int N>
CZ_HD void fwd_avg(float (&x)[N])
{
    constexpr int H = N / 2;
    float s[H], h[H], l[H], d[H];
    uint32_t amax;
    // scalings = 0.5*(x0+x1): binary32 add, exact halving (:159-160)
#pragma unroll
    for (int i = 0; i < H; ++i) s[i] = CZ_MUL(0.5f, CZ_ADD(x[2 * i], x[2 * i + 1]));
    float p0[H], p1[H];
    if (line_split<H>(s, h, l, amax)) {
        p0[0] = st3_fast<P0F>(h[0], h[1], h[2], l[0], l[1], l[2]);
        p1[0] = st3_fast<P1F>(h[0], h[1], h[2], l[0], l[1], l[2]);
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            p0[i] = st3_fast<P0M>(h[i - 1], h[i], h[i + 1], l[i - 1], l[i], l[i + 1]);
            p1[i] = st3_fast<P1M>(h[i - 1], h[i], h[i + 1], l[i - 1], l[i], l[i + 1]);
        }
        p0[H - 1] = st3_fast<P0L>(h[H - 3], h[H - 2], h[H - 1], l[H - 3], l[H - 2], l[H - 1]);
        p1[H - 1] = st3_fast<P1L>(h[H - 3], h[H - 2], h[H - 1], l[H - 3], l[H - 2], l[H - 1]);
    } else {
        p0[0] = st3_any<P0F>(s[0], s[1], s[2]);
        p1[0] = st3_any<P1F>(s[0], s[1], s[2]);
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            p0[i] = st3_any<P0M>(s[i - 1], s[i], s[i + 1]);
            p1[i] = st3_any<P1M>(s[i - 1], s[i], s[i + 1]);
        }
        p0[H - 1] = st3_any<P0L>(s[H - 3], s[H - 2], s[H - 1]);
        p1[H - 1] = st3_any<P1L>(s[H - 3], s[H - 2], s[H - 1]);
    }
    // details = 0.5*((x1-x0) - (p1-p0)), every step in binary32 (:164-176)
#pragma unroll
    for (int i = 0; i < H; ++i)
        d[i] = CZ_MUL(0.5f, CZ_SUB(CZ_SUB(x[2 * i + 1], x[2 * i]), CZ_SUB(p1[i], p0[i])));
#pragma unroll
    for (int i = 0; i < H; ++i) {
        x[i] = s[i];
        x[H + i] = d[i];
    }
}

template <int N>
CZ_HD void inv_avg(float (&x)[N])
{
    constexpr int H = N / 2;
    float s[H], d[H], h[H], l[H], p0[H], p1[H];
    uint32_t amax;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        s[i] = x[i];
        d[i] = x[H + i];
    }
    if (line_split<H>(s, h, l, amax)) {
        p0[0] = st3_fast<P0F>(h[0], h[1], h[2], l[0], l[1], l[2]);
        p1[0] = st3_fast<P1F>(h[0], h[1], h[2], l[0], l[1], l[2]);
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            p0[i] = st3_fast<P0M>(h[i - 1], h[i], h[i + 1], l[i - 1], l[i], l[i + 1]);
            p1[i] = st3_fast<P1M>(h[i - 1], h[i], h[i + 1], l[i - 1], l[i], l[i + 1]);
        }
        p0[H - 1] = st3_fast<P0L>(h[H - 3], h[H - 2], h[H - 1], l[H - 3], l[H - 2], l[H - 1]);
        p1[H - 1] = st3_fast<P1L>(h[H - 3], h[H - 2], h[H - 1], l[H - 3], l[H - 2], l[H - 1]);
    } else {
        p0[0] = st3_any<P0F>(s[0], s[1], s[2]);
        p1[0] = st3_any<P1F>(s[0], s[1], s[2]);
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            p0[i] = st3_any<P0M>(s[i - 1], s[i], s[i + 1]);
            p1[i] = st3_any<P1M>(s[i - 1], s[i], s[i + 1]);
        }
        p0[H - 1] = st3_any<P0L>(s[H - 3], s[H - 2], s[H - 1]);
        p1[H - 1] = st3_any<P1L>(s[H - 3], s[H - 2], s[H - 1]);
    }
    // :187-197
#pragma unroll
    for (int i = 0; i < H; ++i) {
        x[2 * i] = CZ_SUB(p0[i], d[i]);
        x[2 * i + 1] = CZ_ADD(p1[i], d[i]);
    }
}

template <int N>
CZ_HD void fwd_line(float (&x)[N], int wtype)
{
    if (wtype == 1 || wtype == 2) fwd_interp<N>(x, wtype == 2);
    else fwd_avg<N>(x);
}
template <int N>
CZ_HD void inv_line(float (&x)[N], int wtype)
{
    if (wtype == 1 || wtype == 2) inv_interp<N>(x, wtype == 2);
    else inv_avg<N>(x);
}

}  // namespace cz
