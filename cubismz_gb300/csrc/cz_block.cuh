// cz_block.cuh -- shared-memory block machinery of the codec kernels:
// padded block layout, survivor-order runs, their scan, the survivor order
// itself, and record emission. Used by the codec and the refit kernels.
#pragma once
#include "cz_codec.h"
#include "cz_device.cuh"

namespace cz {

constexpr int kNT = 512;
constexpr int kNW = kNT / 32;
constexpr int SY = 33, SZ = 1057;
constexpr int kPadFloats = 32 * SZ;  // 33824
__device__ __forceinline__ int pidx(int x, int y, int z) { return x + SY * y + SZ * z; }

// survivor-order runs ("segments"): coarse (64 entries, always kept), then
// level 8 (7 codes x 16 runs of 4), level 16 (7 x 64 runs of 8), level 32
// (7 x 256 runs of 16)
constexpr int kSeg8 = 112, kSeg16 = 448, kSeg32 = 1792;
constexpr int kSegBase8 = 1, kSegBase16 = kSegBase8 + kSeg8, kSegBase32 = kSegBase16 + kSeg16;
constexpr int kSegs = kSegBase32 + kSeg32;  // 2353

// shared memory map (bytes)
constexpr int kSmBlock = 0;
constexpr int kSmMask = ((kPadFloats * 4 + 15) / 16) * 16;  // 4096 B, u32 words
constexpr int kSmSeg32 = kSmMask + kMaskBytes;              // u16 x 1792
constexpr int kSmSeg16 = kSmSeg32 + kSeg32 * 2;             // u8 x 448
constexpr int kSmSeg8 = kSmSeg16 + kSeg16;                  // u8 x 112
constexpr int kSmOff = ((kSmSeg8 + kSeg8 + 15) / 16) * 16;  // int x kSegs
constexpr int kSmWarp = ((kSmOff + 4 * (kSegs + 1) + 15) / 16) * 16;
constexpr int kSmBytes = kSmWarp + 4 * 64;

struct BlockRef {
    const CzField *f;
    int bx, by, bz;
};

__device__ __forceinline__ BlockRef locate(const CzField *fields, int nfields, long long g)
{
    int lo = 0, hi = nfields - 1;
    while (lo < hi) {  // last field with block0 <= g
        const int mid = (lo + hi + 1) >> 1;
        if (fields[mid].block0 <= g) lo = mid;
        else hi = mid - 1;
    }
    const CzField *f = &fields[lo];
    const long long b = g - f->block0;
    const int nbx = f->nx >> 5, nby = f->ny >> 5;
    BlockRef r;
    r.f = f;
    r.bx = (int)(b % nbx);
    r.by = (int)((b / nbx) % nby);
    r.bz = (int)(b / ((long long)nbx * nby));
    return r;
}

__device__ __forceinline__ size_t row_offset(const BlockRef &r, int y, int z)
{
    const CzField &f = *r.f;
    return ((size_t)(r.bz * 32 + z) * f.ny + (size_t)(r.by * 32 + y)) * f.nx + (size_t)r.bx * 32;
}

// Rows (y, z) and (y, z+16) of a block, y = tid&31, z = tid>>5: the two x
// lines this thread transforms first.
__device__ __forceinline__ void load_rows(const BlockRef &r, float4 (&pf)[16])
{
    const int y = threadIdx.x & 31, z = threadIdx.x >> 5;
    const float4 *r0 = reinterpret_cast<const float4 *>(r.f->data + row_offset(r, y, z));
    const float4 *r1 = reinterpret_cast<const float4 *>(r.f->data + row_offset(r, y, z + 16));
#pragma unroll
    for (int k = 0; k < 8; ++k) pf[k] = __ldg(r0 + k);
#pragma unroll
    for (int k = 0; k < 8; ++k) pf[8 + k] = __ldg(r1 + k);
}

template <int N>
__device__ __forceinline__ unsigned keep_bits(const float (&v)[N], float eps)
{
    unsigned b = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) b |= (unsigned)(fabsf(v[j]) > eps) << j;  // FullWaveletTransform.h:84
    return b;
}

// ------------------------------------------------------------------ sweeps
// Line l of a sweep along AXIS over the [0,N)^3 corner: the two other
// coordinates are (l % N, l / N), lowest first.
template <int N, int AXIS>
__device__ __forceinline__ int line_base(int l)
{
    const int a = l % N, c = l / N;
    if (AXIS == 0) return pidx(0, a, c);
    if (AXIS == 1) return pidx(a, 0, c);
    return pidx(a, c, 0);
}
template <int AXIS>
__host__ __device__ constexpr int stride() { return AXIS == 0 ? 1 : (AXIS == 1 ? SY : SZ); }

template <int N, int AXIS>
__device__ __forceinline__ void ld_line(const float *sb, int base, float (&v)[N])
{
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = sb[base + j * stride<AXIS>()];
}
template <int N, int AXIS>
__device__ __forceinline__ void st_line(float *sb, int base, const float (&v)[N])
{
#pragma unroll
    for (int j = 0; j < N; ++j) sb[base + j * stride<AXIS>()] = v[j];
}

template <int N, int AXIS, bool FWD, int KIND>
__device__ __forceinline__ void sweep(float *sb)
{
    for (int l = threadIdx.x; l < N * N; l += kNT) {
        const int base = line_base<N, AXIS>(l);
        float v[N];
        ld_line<N, AXIS>(sb, base, v);
        if (FWD) line_fwd<N, KIND>(v);
        else line_inv<N, KIND>(v);
        st_line<N, AXIS>(sb, base, v);
    }
}

// ------------------------------------------------------------ thresholding
struct Shared {
    float *sb;
    uint32_t *mask32;
    uint16_t *seg32;
    uint8_t *seg16, *seg8;
    int *off, *warp;
};

__device__ __forceinline__ Shared carve(unsigned char *smem)
{
    Shared s;
    s.sb = reinterpret_cast<float *>(smem + kSmBlock);
    s.mask32 = reinterpret_cast<uint32_t *>(smem + kSmMask);
    s.seg32 = reinterpret_cast<uint16_t *>(smem + kSmSeg32);
    s.seg16 = smem + kSmSeg16;
    s.seg8 = smem + kSmSeg8;
    s.off = reinterpret_cast<int *>(smem + kSmOff);
    s.warp = reinterpret_cast<int *>(smem + kSmWarp);
    return s;
}

// Level-32 z line (x,y): positional word y*32+x holds its bits z (px = z,
// py = x, pz = y); runs are z<16 (octant code with px bit 0) and z>=16.
__device__ __forceinline__ void emit32(const Shared &s, int x, int y, unsigned kb)
{
    const int chi = 1 | ((x >= 16) << 1) | ((y >= 16) << 2);
    const int sub = ((y & 15) << 4) | (x & 15);
    s.seg32[(chi - 1) * 256 + sub] = (uint16_t)(kb >> 16);
    const int w = x + 32 * y;
    if (chi > 1) {
        s.seg32[(chi - 2) * 256 + sub] = (uint16_t)kb;
        s.mask32[w] = kb;
    } else {
        reinterpret_cast<uint16_t *>(s.mask32)[2 * w + 1] = (uint16_t)(kb >> 16);
    }
}
// Level-16 y line (x,z): positional word x*32+z holds its bits y (px = y,
// py = z, pz = x); runs are y<8 and y>=8.
__device__ __forceinline__ void emit16(const Shared &s, int x, int z, unsigned kb)
{
    const int chi = 1 | ((z >= 8) << 1) | ((x >= 8) << 2);
    const int sub = ((x & 7) << 3) | (z & 7);
    s.seg16[(chi - 1) * 64 + sub] = (uint8_t)(kb >> 8);
    const int w = z + 32 * x;
    if (chi > 1) {
        s.seg16[(chi - 2) * 64 + sub] = (uint8_t)kb;
        reinterpret_cast<uint16_t *>(s.mask32)[2 * w] = (uint16_t)kb;
    } else {
        reinterpret_cast<uint8_t *>(s.mask32)[4 * w + 1] = (uint8_t)(kb >> 8);
    }
}
// Level-8 x line (y,z): positional word z*32+y holds its bits x; the coarse
// 4^3 corner is always kept (FullWaveletTransform.h:165-168).
__device__ __forceinline__ void emit8(const Shared &s, int y, int z, unsigned kb)
{
    if (y < 4 && z < 4) kb |= 0xFu;
    const int chi = 1 | ((y >= 4) << 1) | ((z >= 4) << 2);
    const int sub = ((z & 3) << 2) | (y & 3);
    s.seg8[(chi - 1) * 16 + sub] = (uint8_t)(kb >> 4);
    if (chi > 1) s.seg8[(chi - 2) * 16 + sub] = (uint8_t)(kb & 0xF);
    reinterpret_cast<uint8_t *>(s.mask32)[4 * (y + 32 * z)] = (uint8_t)kb;
}

__device__ __forceinline__ int seg_count(const Shared &s, int i)
{
    if (i < kSegBase8) return 64;
    if (i < kSegBase16) return __popc(s.seg8[i - kSegBase8]);
    if (i < kSegBase32) return __popc(s.seg16[i - kSegBase16]);
    return __popc(s.seg32[i - kSegBase32]);
}

// Exclusive scan of the run counts into s.off; returns the survivor total.
__device__ __forceinline__ int scan_segments(const Shared &s)
{
    constexpr int PER = (kSegs + kNT - 1) / kNT;  // 5
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i0 = threadIdx.x * PER;
    int c[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        c[k] = (i0 + k < kSegs) ? seg_count(s, i0 + k) : 0;
        sum += c[k];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s.warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int v = lane < kNW ? s.warp[lane] : 0;
        int w = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < kNW) s.warp[32 + lane] = w - v;
        if (lane == kNW - 1) s.warp[32 + kNW] = w;
    }
    __syncthreads();
    int run = s.warp[32 + warp] + incl - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        if (i0 + k < kSegs) s.off[i0 + k] = run;
        run += c[k];
    }
    const int total = s.warp[32 + kNW];
    __syncthreads();
    return total;
}

// Survivor-order slot -> (physical position, run mask, bit within the run,
// run offset). The 32 slots of a chunk share their level.
struct Slot {
    int pos;
    unsigned mask;
    int e;
    int off;
};
__device__ __forceinline__ Slot slot_of(const Shared &s, int sidx)
{
    Slot r;
    if (sidx < 64) {  // coarse, z,y,x order (FullWaveletTransform.h:170-173)
        r.pos = pidx(sidx & 3, (sidx >> 2) & 3, sidx >> 4);
        r.mask = 0xffffffffu;
        r.e = 0;
        r.off = sidx;
        return r;
    }
    if (sidx < 512) {  // level 8: runs of 4 along x
        const int q = sidx - 64, seg = q >> 2, e = q & 3, c = (seg >> 4) + 1;
        r.pos = pidx(4 * (c & 1) + e, 4 * ((c >> 1) & 1) + (seg & 3), 4 * (c >> 2) + ((seg >> 2) & 3));
        r.mask = s.seg8[seg];
        r.e = e;
        r.off = s.off[kSegBase8 + seg];
        return r;
    }
    if (sidx < 4096) {  // level 16: runs of 8 along y
        const int q = sidx - 512, seg = q >> 3, e = q & 7, c = (seg >> 6) + 1;
        r.pos = pidx(8 * (c >> 2) + ((seg >> 3) & 7), 8 * (c & 1) + e, 8 * ((c >> 1) & 1) + (seg & 7));
        r.mask = s.seg16[seg];
        r.e = e;
        r.off = s.off[kSegBase16 + seg];
        return r;
    }
    // level 32: runs of 16 along z
    const int q = sidx - 4096, seg = q >> 4, e = q & 15, c = (seg >> 8) + 1;
    r.pos = pidx(16 * ((c >> 1) & 1) + (seg & 15), 16 * (c >> 2) + ((seg >> 4) & 15), 16 * (c & 1) + e);
    r.mask = s.seg32[seg];
    r.e = e;
    r.off = s.off[kSegBase32 + seg];
    return r;
}

// ------------------------------------------------------------------ decode
// Run masks from the positional mask words (the inverse of emit32/16/8).
__device__ __forceinline__ void runs_from_mask(const Shared &s)
{
    for (int i = threadIdx.x; i < kSeg32; i += kNT) {
        const int c = (i >> 8) + 1, sub = i & 255;
        const int x = 16 * ((c >> 1) & 1) + (sub & 15), y = 16 * (c >> 2) + (sub >> 4);
        s.seg32[i] = (uint16_t)(s.mask32[x + 32 * y] >> (16 * (c & 1)));
    }
    for (int i = threadIdx.x; i < kSeg16; i += kNT) {
        const int c = (i >> 6) + 1, sub = i & 63;
        const int x = 8 * (c >> 2) + (sub >> 3), z = 8 * ((c >> 1) & 1) + (sub & 7);
        s.seg16[i] = (uint8_t)(s.mask32[z + 32 * x] >> (8 * (c & 1)));
    }
    for (int i = threadIdx.x; i < kSeg8; i += kNT) {
        const int c = (i >> 4) + 1, sub = i & 15;
        const int y = 4 * ((c >> 1) & 1) + (sub & 3), z = 4 * (c >> 2) + (sub >> 2);
        s.seg8[i] = (uint8_t)((s.mask32[y + 32 * z] >> (4 * (c & 1))) & 0xF);
    }
}

struct Payload {
    const uint8_t *p;
    int c;  // byte-plane stride (reshuffle3's n/4, WaveletCompressor.cpp:80)
    bool shuffle;
    __device__ __forceinline__ float get(int k) const
    {
        if (shuffle)
            return __uint_as_float((uint32_t)p[k] | ((uint32_t)p[c + k] << 8) | ((uint32_t)p[2 * c + k] << 16) |
                                   ((uint32_t)p[3 * c + k] << 24));
        return __uint_as_float(reinterpret_cast<const uint32_t *>(p)[k]);
    }
};

// Value at bit e of run `seg` (global run index): its survivor or zero.
__device__ __forceinline__ float run_value(const Shared &s, const Payload &pl, unsigned mask, int seg, int e)
{
    if (!((mask >> e) & 1u)) return 0.f;
    return pl.get(s.off[seg] + __popc(mask & ((1u << e) - 1u)));
}

// Record emission for block g once its coefficients sit in s.sb and its run
// masks in s.seg*/s.mask32: [int32 nbytes][mask][survivors in the reference
// order, zero-bits applied, byte planes when shuffling]
// (WaveletCompressor.cpp:152-182, SerializerIO_WaveletCompression_MPI_Simple.h:236-240).
__device__ __forceinline__ void emit_record(const Shared &s, long long g, uint32_t zmask, int shuffle, uint8_t *stage,
                                            int *rec_bytes)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // ---- offsets of every run, record header and mask
    const int S = scan_segments(s);
    const int nb = kMaskBytes + 4 * S;
    uint8_t *slot = stage + (size_t)g * kSlotBytes;
    if (threadIdx.x == 0) {
        *reinterpret_cast<int *>(slot) = nb;
        rec_bytes[g] = nb;
    }
    for (int i = threadIdx.x; i < kMaskBytes / 4; i += kNT)
        reinterpret_cast<uint32_t *>(slot + 4)[i] = s.mask32[i];
    // ---- survivors in the reference order, zero-bits, byte planes
    uint8_t *pay = slot + 4 + kMaskBytes;
    for (int ch = warp; ch < 1024; ch += kNW) {
        const Slot t = slot_of(s, ch * 32 + lane);
        if ((t.mask >> t.e) & 1u) {
            const int k = t.off + __popc(t.mask & ((1u << t.e) - 1u));
            const uint32_t u = __float_as_uint(s.sb[t.pos]) & zmask;
            if (shuffle) {
                pay[k] = (uint8_t)u;
                pay[S + k] = (uint8_t)(u >> 8);
                pay[2 * S + k] = (uint8_t)(u >> 16);
                pay[3 * S + k] = (uint8_t)(u >> 24);
            } else {
                reinterpret_cast<uint32_t *>(pay)[k] = u;
            }
        }
    }
}

}  // namespace cz
