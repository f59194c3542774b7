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
constexpr int kSmStage = kSmWarp + 4 * 64;                  // float x 512 per warp
constexpr int kStagePerWarp = 512;                          // survivors of 32 runs
constexpr int kSmBytes = kSmStage + 4 * kStagePerWarp * (kNT / 32);

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
    float *stage;
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
    s.stage = reinterpret_cast<float *>(smem + kSmStage);
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

// Run r (1 .. kSegs-1) of the survivor order: its keep mask, and the
// physical position of its bit e (the reference's order,
// FullWaveletTransform.h:63-93: per level 8, 16, 32 the octant codes 1..7,
// each in z,y,x order; cz_layout.cuh gives the position maps).
__device__ __forceinline__ unsigned run_mask(const Shared &s, int r)
{
    if (r < kSegBase16) return s.seg8[r - kSegBase8];
    if (r < kSegBase32) return s.seg16[r - kSegBase16];
    return s.seg32[r - kSegBase32];
}
// Physical position of bit e of run r: base + e * stride.
__device__ __forceinline__ void run_geom(int r, int &base, int &stride)
{
    if (r < kSegBase16) {  // level 8: runs of 4 along x
        const int q = r - kSegBase8, c = (q >> 4) + 1;
        base = pidx(4 * (c & 1), 4 * ((c >> 1) & 1) + (q & 3), 4 * (c >> 2) + ((q >> 2) & 3));
        stride = 1;
    } else if (r < kSegBase32) {  // level 16: runs of 8 along y
        const int q = r - kSegBase16, c = (q >> 6) + 1;
        base = pidx(8 * (c >> 2) + ((q >> 3) & 7), 8 * (c & 1), 8 * ((c >> 1) & 1) + (q & 7));
        stride = SY;
    } else {  // level 32: runs of 16 along z
        const int q = r - kSegBase32, c = (q >> 8) + 1;
        base = pidx(16 * ((c >> 1) & 1) + (q & 15), 16 * (c >> 2) + ((q >> 4) & 15), 16 * (c & 1));
        stride = SZ;
    }
}

// Survivors of a block in stream order, 32 runs at a time per warp (one run
// per lane; the survivors of consecutive runs are consecutive in the
// stream). The coarse 4^3 block comes first, always kept, in z,y,x order.
// Needs s.off from scan_segments and S, the survivor total.
//   emit: every lane copies its run's survivors from the block into the
//         warp's stage, then the warp hands them out in stream order,
//         put(k, value) with k consecutive across the warp;
//   load: the warp fetches the group's values in stream order,
//         get(k) with k consecutive across the warp, into the stage; every
//         lane then places its run's survivors in the block.
template <class Put>
__device__ __forceinline__ void emit_survivors(const Shared &s, int S, Put &&put)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stg = s.stage + warp * kStagePerWarp;
    if (threadIdx.x < 64) {
        const int t = threadIdx.x;
        put(t, s.sb[pidx(t & 3, (t >> 2) & 3, t >> 4)]);
    }
    for (int r0 = kSegBase8 + 32 * warp; r0 < kSegs; r0 += 32 * kNW) {
        const int r = r0 + lane;
        const unsigned m = r < kSegs ? run_mask(s, r) : 0u;
        const int o = r < kSegs ? s.off[r] : S;
        const int first = __shfl_sync(0xffffffffu, o, 0);
        const int total = __shfl_sync(0xffffffffu, o + __popc(m), 31) - first;
        if (total == 0) continue;
        int base = 0, stride = 0;
        if (r < kSegs) run_geom(r, base, stride);
        int i = o - first;
        for (unsigned mm = m; mm; mm &= mm - 1) stg[i++] = s.sb[base + (__ffs(mm) - 1) * stride];
        __syncwarp();
        for (int b = lane; b < total; b += 32) put(first + b, stg[b]);
        __syncwarp();
    }
}
template <class Get>
__device__ __forceinline__ void load_survivors(const Shared &s, int S, Get &&get)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stg = s.stage + warp * kStagePerWarp;
    if (threadIdx.x < 64) {
        const int t = threadIdx.x;
        s.sb[pidx(t & 3, (t >> 2) & 3, t >> 4)] = get(t);
    }
    for (int r0 = kSegBase8 + 32 * warp; r0 < kSegs; r0 += 32 * kNW) {
        const int r = r0 + lane;
        const unsigned m = r < kSegs ? run_mask(s, r) : 0u;
        const int o = r < kSegs ? s.off[r] : S;
        const int first = __shfl_sync(0xffffffffu, o, 0);
        const int total = __shfl_sync(0xffffffffu, o + __popc(m), 31) - first;
        if (total > 0) {
            for (int b = lane; b < total; b += 32) stg[b] = get(first + b);
            __syncwarp();
        }
        int base = 0, stride = 0;
        if (r < kSegs) run_geom(r, base, stride);
        int i = o - first;
        // every place of the run: its survivor or zero (the runs and the
        // coarse corner cover the whole block, so no separate zeroing)
        const int len = r < kSegBase16 ? 4 : (r < kSegBase32 ? 8 : 16);
        if (r < kSegs)
            for (int e = 0; e < len; ++e) s.sb[base + e * stride] = ((m >> e) & 1u) ? stg[i++] : 0.f;
        __syncwarp();
    }
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

// n bytes from p into L2, one 128-byte line per thread and step, by
// threads t of nt (a hint: nothing is read into registers)
__device__ __forceinline__ void prefetch_l2_span(const uint8_t *p, int n, int t, int nt)
{
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)127;
    const uintptr_t a1 = reinterpret_cast<uintptr_t>(p) + (uintptr_t)(n > 0 ? n : 0);
    for (uintptr_t a = a0 + 128 * (uintptr_t)t; a < a1; a += 128 * (uintptr_t)nt)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

// A record's bytes into L2 (byte planes 1 and 2 from q12 when the LZ4 stage
// left them in its input) by threads t of nt.
__device__ __forceinline__ void prefetch_record(const uint8_t *slot, int nb, const uint8_t *q12, int t, int nt)
{
    const uint8_t *pay = slot + 4 + kMaskBytes;
    const int np = nb - kMaskBytes, c4 = np / 4;
    if (q12) {
        prefetch_l2_span(slot, 4 + kMaskBytes + c4, t, nt);
        prefetch_l2_span(q12, 2 * c4, t, nt);
        prefetch_l2_span(pay + 3 * c4, np - 3 * c4, t, nt);
    } else {
        prefetch_l2_span(slot, 4 + nb, t, nt);
    }
}

struct Payload {
    const uint8_t *p;
    const uint8_t *q;  // byte planes 1 and 2 (p + c, or where the LZ4 stage left them)
    int c;             // byte-plane stride (reshuffle3's n/4, WaveletCompressor.cpp:80)
    bool shuffle;
    __device__ __forceinline__ float get(int k) const
    {
        if (shuffle)
            return __uint_as_float((uint32_t)p[k] | ((uint32_t)q[k] << 8) | ((uint32_t)q[c + k] << 16) |
                                   ((uint32_t)p[3 * c + k] << 24));
        return __uint_as_float(reinterpret_cast<const uint32_t *>(p)[k]);
    }
};

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
    emit_survivors(s, S, [&](int k, float v) {
        const uint32_t u = __float_as_uint(v) & zmask;
        if (shuffle) {
            pay[k] = (uint8_t)u;
            pay[S + k] = (uint8_t)(u >> 8);
            pay[2 * S + k] = (uint8_t)(u >> 16);
            pay[3 * S + k] = (uint8_t)(u >> 24);
        } else {
            reinterpret_cast<uint32_t *>(pay)[k] = u;
        }
    });
}

}  // namespace cz
