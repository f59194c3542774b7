// cz_lz4rec.cu -- the LZ4 stage of block-record chunks, parsed region by
// region.
//
// A chunk of block records holds, per record, three runs of bytes with
// their own statistics: the record header and significance mask, byte
// plane 0 (low mantissa bits) and byte plane 3 (sign and exponent) compress;
// planes 1 and 2 (the middle mantissa bits) do not (shuffle3's planes,
// WaveletCompressor.cpp:55-73). Greedy LZ4 parses of the three regions,
// each with its own history, compress a record as well as one parse of the
// whole chunk, so every region is parsed by its own warp, independently:
//
//   lz4_region_kernel  one warp per region. The region's bytes stream
//       through a 4 KB ring in shared memory, two windows ahead of the
//       parse (loads issued a window before they are stored), so every
//       candidate check and literal copy reads shared memory. Per window of
//       512 positions:
//         probe -- 4 consecutive positions per lane per step: hash of the
//                  4 bytes (LZ4's multiplicative hash, lz4.c:515), lookup
//                  and insert in a 2048-entry table of 16-bit positions,
//                  the candidate checked against the ring and its match
//                  length measured up to 8 bytes; offsets up to 3072;
//         walk  -- lane k parses positions [16k, 16k+16) of the window
//                  greedily (the reference's parse: take the match at the
//                  cursor, jump past it, else step one byte, lz4.c:556-672);
//         merge -- the exact greedy parse of the window: a lane whose entry
//                  point (where the parse leaves the lanes below) is not on
//                  its own walk walks again from there; repeated until no
//                  lane's exit moves;
//         emit  -- sizes, a warp scan, every lane writes its sequences into
//                  a shared-memory stage that the warp flushes with word
//                  stores.
//       The region's output is its sequences from its start a: the first
//       sequence's literal run starts at a, and the literals after its last
//       match are left to the next region.
//   lz4_region_sizes   per chunk, the size of the joined LZ4 block.
//   lz4_stitch_kernel  one warp per chunk joins the regions: each region's
//       first sequence gets its literal run extended back to the previous
//       region's last match (a new token and length bytes, the literal
//       bytes from the records -- the incompressible planes among them),
//       then the region's bytes follow; the block ends with the last
//       literals. The result is one LZ4 block per chunk in the legacy
//       format that LZ4_uncompress_unknownOutputSize reads (lz4.c:802-905):
//       minimum match 4, offsets below 64 KiB, the last match starting at
//       least 12 bytes and ending at least 5 bytes before the end
//       (lz4.c:177-204).
#include "cz_codec.h"
#include "cz_device.cuh"

namespace cz {
namespace lzr {

constexpr int kW = 512;                  // positions per window
constexpr int kSub = kW / 32;            // walk positions per lane
constexpr int kRing = 4096;              // bytes of history in shared memory
constexpr int kRingWords = kRing / 4;
constexpr int kMaxOff = kRing - 2 * kW;  // candidate bytes stay in the ring
constexpr int kHLog = 11;
constexpr int kStage = 1024;             // staged output bytes per window
constexpr int kMaxSeq = kSub / 4;        // sequences a lane's walk can start
constexpr int kWarps = 2;                // regions (warps) per CTA
constexpr unsigned kFull = 0xffffffffu;

struct Smem {
    uint32_t ring[kRingWords];
    uint16_t table[1 << kHLog];
    uint16_t info[kW];             // valid | (len-4) << 12 | offset; 0: none
    uint32_t seq[kMaxSeq][32];     // start - window | offset << 16
    uint32_t slen[kMaxSeq][32];    // match length
    uint32_t stage[kStage / 4 + 4];
};

__device__ __forceinline__ uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHLog); }
__device__ __forceinline__ uint32_t fsr(uint32_t lo, uint32_t hi, uint32_t sh)
{
    return sh ? __funnelshift_r(lo, hi, sh) : lo;
}
__device__ __forceinline__ int ext_bytes(int n) { return n >= 15 ? (n - 15) / 255 + 1 : 0; }

// 4 bytes of the region at byte position x, from the ring
__device__ __forceinline__ uint32_t ring4(const uint32_t *ring, int x)
{
    const int wi = x >> 2;
    return fsr(ring[wi & (kRingWords - 1)], ring[(wi + 1) & (kRingWords - 1)], (uint32_t)(x & 3) * 8);
}
// 32-bit little-endian word at any byte address of global memory
__device__ __forceinline__ uint32_t gld4(const uint8_t *p)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    return fsr(__ldg(w), __ldg(w + 1), (uint32_t)(a & 3) * 8);
}

// Match length from (p, c) starting `known` bytes in, up to lim - p, from
// global memory (matches of more than 8 bytes, about 2 % of them).
__device__ int extend(const uint8_t *src, int p, int c, int known, int lim)
{
    int len = known;
    while (p + len < lim) {
        const uint32_t x = gld4(src + p + len) ^ gld4(src + c + len);
        if (x) {
            len += (__ffs(x) - 1) >> 3;
            break;
        }
        len += 4;
    }
    return len < lim - p ? len : lim - p;
}

__device__ __forceinline__ uint8_t *put_ext(uint8_t *d, int n)
{
    for (; n >= 255; n -= 255) *d++ = 255;
    *d++ = (uint8_t)n;
    return d;
}

// Literal bytes [from, from+n) into d: from the ring when the ring still
// holds them, else from global memory.
__device__ __forceinline__ void copy_lits(uint8_t *d, const uint32_t *ring, bool in_ring, const uint8_t *src,
                                          int from, int n)
{
    for (int i = 0; i < n; i += 4) {
        const uint32_t v = in_ring ? ring4(ring, from + i) : gld4(src + from + i);
        d[i] = (uint8_t)v;
        if (i + 1 < n) d[i + 1] = (uint8_t)(v >> 8);
        if (i + 2 < n) d[i + 2] = (uint8_t)(v >> 16);
        if (i + 3 < n) d[i + 3] = (uint8_t)(v >> 24);
    }
}

// Greedy walk of lane positions [from, e) of window w; the lane's sequences
// go to s.seq/s.slen, `vis` gets a bit per visited position (relative to
// sl), and the exit (first position past the lane's parse) is returned.
__device__ __forceinline__ int walk(Smem &s, const uint8_t *src, int w, int sl, int from, int e, int lim, int lane,
                                    int &ns, uint32_t &vis)
{
    ns = 0;
    vis = 0;
    int q = from;
    while (q < e) {
        vis |= 1u << (q - sl);
        const uint32_t inf = s.info[q - w];
        if (inf) {
            int len = (int)((inf >> 12) & 7) + 4;
            const int o = (int)(inf & 0xfff);
            if (len == 8 && q + 8 < lim) len = extend(src, q, q - o, 8, lim);
            s.seq[ns][lane] = (uint32_t)(q - w) | ((uint32_t)o << 16);
            s.slen[ns][lane] = (uint32_t)len;
            ++ns;
            q += len;
        } else {
            ++q;
        }
    }
    return q;
}

// Output byte area of region `ridx` (0, 1, ...) starting at chunk position
// a: non-overlapping for regions in position order, each at least
// n + n/8 + 47 bytes for a region of n bytes (an LZ4 parse of n bytes
// writes at most n*16/15 + 4, length bytes included).
__device__ __forceinline__ long long area_off(int a, int ridx)
{
    return (((long long)a + (a >> 3) + 15) & ~15LL) + 64LL * ridx;
}

// One region per warp: regions (c, j, k) of chunk c, record j of the chunk,
// kind k (0: record header and mask; 1: byte plane 0, or the whole payload
// without shuffle; 2: byte plane 3).
__global__ void __launch_bounds__(kWarps * 32)
lz4_region_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  const int *rec_bytes, const long long *blk_dst, long long nblocks, int bpc, int shuffle,
                  uint8_t *__restrict__ out, const long long *out_off, LzRegion *reg)
{
    extern __shared__ __align__(16) unsigned char lzr_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Smem &s = reinterpret_cast<Smem *>(lzr_smem)[wib];
    const long long nreg = (long long)nchunks * bpc * 3;
    for (long long ri = (long long)blockIdx.x * kWarps + wib; ri < nreg; ri += (long long)gridDim.x * kWarps) {
        const int c = (int)(ri / (3 * bpc));
        const int j = (int)((ri / 3) % bpc), k = (int)(ri % 3);
        const long long g = (long long)c * bpc + j;
        const uint8_t *src = in + in_off[c];
        const int L = in_len[c];
        int a = L, b = L;
        if (g < nblocks) {
            const int rb = blk_dst ? (int)(blk_dst[g] - in_off[c]) : 0;
            const int nb = rec_bytes[g];
            const int S = (nb - kMaskBytes) / 4;
            if (k == 0) {
                a = rb;
                b = rb + 4 + kMaskBytes;
            } else if (shuffle) {
                a = rb + 4 + kMaskBytes + (k == 1 ? 0 : 3 * S);
                b = a + S;
            } else if (k == 1) {
                a = rb + 4 + kMaskBytes;
                b = rb + 4 + nb;
            } else {
                a = b = rb + 4 + nb;
            }
        }
        const int ridx = j * 3 + k;
        uint8_t *dst = out + out_off[c] + area_off(a, ridx);
        const int n = b - a;
        const int cap = n + (n >> 3) + 40;
        const int lim = min(b, L - 5);        // matches end at or before
        const int plim = min(b - 4, L - 12);  // and start at or before
        int first_st = -1, first_hdr = 0, anchor = a, op = 0;
        bool ovf = false;
        if (plim >= a) {
            for (int i = lane; i < (1 << kHLog) / 2; i += 32) reinterpret_cast<uint32_t *>(s.table)[i] = kFull;
            const int w0 = a & ~3;
            // the ring starts with the region's first two windows
#pragma unroll
            for (int q = 0; q < 2 * kW / 128; ++q) {
                const int pos = w0 + 128 * q + 4 * lane;
                s.ring[(pos >> 2) & (kRingWords - 1)] =
                    pos <= L ? __ldg(reinterpret_cast<const uint32_t *>(src + pos)) : 0u;
            }
            __syncwarp();
            int entry = a;  // where the parse enters the next window
            int pend = 0;   // bytes of a partial output word held in s.stage[0]
            uint32_t *d32 = reinterpret_cast<uint32_t *>(dst);
            uint8_t *stg = reinterpret_cast<uint8_t *>(s.stage);
            for (int w = w0; w <= plim; w += kW) {
                // the window after next: loaded now, stored into the ring at the end
                uint32_t pf[kW / 128];
#pragma unroll
                for (int q = 0; q < kW / 128; ++q) {
                    const int pos = w + 2 * kW + 128 * q + 4 * lane;
                    pf[q] = pos <= L ? __ldg(reinterpret_cast<const uint32_t *>(src + pos)) : 0u;
                }
                if (entry < w + kW) {
                    // ---- probe
#pragma unroll 1
                    for (int st = 0; st < kW / 128; ++st) {
                        const int p0 = w + 128 * st + 4 * lane;
                        const int wi = p0 >> 2;
                        const uint32_t q0 = s.ring[wi & (kRingWords - 1)], q1 = s.ring[(wi + 1) & (kRingWords - 1)],
                                       q2 = s.ring[(wi + 2) & (kRingWords - 1)];
                        uint32_t v[4], h[4], e[4];
#pragma unroll
                        for (int jj = 0; jj < 4; ++jj) {
                            v[jj] = fsr(q0, q1, 8 * jj);
                            h[jj] = hash4(v[jj]);
                            e[jj] = s.table[h[jj]];
                        }
                        __syncwarp();
#pragma unroll
                        for (int jj = 0; jj < 4; ++jj) {
                            const int p = p0 + jj;
                            if (p >= a && p <= plim) s.table[h[jj]] = (uint16_t)p;
                        }
                        __syncwarp();
#pragma unroll
                        for (int jj = 0; jj < 4; ++jj) {
                            const int p = p0 + jj;
                            const int o = (int)(((uint32_t)p - e[jj]) & 0xffffu);
                            const int cnd = p - o;
                            uint32_t inf = 0;
                            if (p >= a && p <= plim && o >= 1 && o <= kMaxOff && cnd >= a) {
                                if (ring4(s.ring, cnd) == v[jj]) {
                                    const uint32_t x = fsr(q1, q2, 8 * jj) ^ ring4(s.ring, cnd + 4);
                                    int len = x ? 4 + ((__ffs(x) - 1) >> 3) : 8;
                                    len = min(len, lim - p);
                                    if (len >= 4) inf = 0x8000u | ((uint32_t)(len - 4) << 12) | (uint32_t)o;
                                }
                            }
                            s.info[p - w] = (uint16_t)inf;
                        }
                    }
                    __syncwarp();
                    // ---- walk: lane positions [sl, el)
                    const int sl = w + kSub * lane, el = sl + kSub;
                    int ns, start = sl;
                    uint32_t vis;
                    // Xw: exit of the lane's current walk; X: where the parse
                    // leaves the lane (Xw, or the entry when the parse passes
                    // over the lane)
                    int Xw = walk(s, src, w, sl, sl, el, lim, lane, ns, vis);
                    int X = Xw;
                    // ---- merge: the entry E of a lane is the exit of the lane below
                    int E = entry;
#pragma unroll 1
                    for (int it = 0; it < 34; ++it) {
                        const int up = __shfl_up_sync(kFull, X, 1);
                        E = lane ? up : entry;
                        int nX;
                        if (E >= el) {
                            nX = E;  // the parse passes over this lane
                        } else if (E >= start && ((vis >> (E - sl)) & 1u)) {
                            nX = Xw;  // E is on the lane's walk
                        } else {
                            start = E;  // not on the lane's walk: walk again from E
                            Xw = walk(s, src, w, sl, E, el, lim, lane, ns, vis);
                            nX = Xw;
                        }
                        const bool moved = nX != X;
                        X = nX;
                        if (!__any_sync(kFull, moved)) break;
                    }
                    // ---- emit: kept sequences start at or after E
                    int nk = 0, kept_end = 0, my_first = 0;
                    for (int i = 0; i < ns; ++i) {
                        const int st = w + (int)(s.seq[i][lane] & 0xffffu);
                        if (E < el && st >= E) {
                            if (!nk) my_first = st;
                            ++nk;
                            kept_end = st + (int)s.slen[i][lane];
                        }
                    }
                    const unsigned has = __ballot_sync(kFull, nk > 0);
                    const unsigned lower = has & cz::lanemask_lt();
                    const int lsrc = lower ? 31 - __clz(lower) : 0;
                    const int lend = __shfl_sync(kFull, kept_end, lsrc);
                    const int lf0 = lower ? lend : anchor;
                    int bytes = 0;
                    {
                        int lf = lf0;
                        for (int i = 0; i < ns; ++i) {
                            const int st = w + (int)(s.seq[i][lane] & 0xffffu);
                            if (!(E < el && st >= E)) continue;
                            const int lit = st - lf, ml = (int)s.slen[i][lane] - 4;
                            bytes += 1 + ext_bytes(lit) + lit + 2 + ext_bytes(ml);
                            lf = st + ml + 4;
                        }
                    }
                    int incl = bytes;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int t = __shfl_up_sync(kFull, incl, o);
                        if (lane >= o) incl += t;
                    }
                    const int T = __shfl_sync(kFull, incl, 31);
                    if (has) {
                        if (first_st < 0) {
                            const int f = __ffs(has) - 1;
                            first_st = __shfl_sync(kFull, my_first, f);
                            first_hdr = 1 + ext_bytes(first_st - a);
                        }
                        const int top = 31 - __clz(has);
                        const int new_anchor = __shfl_sync(kFull, kept_end, top);
                        if (op + T + 8 > cap) {
                            ovf = true;
                            break;
                        }
                        const bool staged = pend + T <= kStage;
                        const int ring_lo = w + 2 * kW - kRing;
                        if (!staged) {
                            if (pend && lane == 0) d32[(op - pend) >> 2] = s.stage[0];
                            __syncwarp();
                        }
                        uint8_t *d = staged ? stg + pend + (incl - bytes) : dst + op + (incl - bytes);
                        int lf = lf0;
                        for (int i = 0; i < ns; ++i) {
                            const int st = w + (int)(s.seq[i][lane] & 0xffffu);
                            if (!(E < el && st >= E)) continue;
                            const int lit = st - lf, ml = (int)s.slen[i][lane] - 4;
                            const int off = (int)(s.seq[i][lane] >> 16);
                            *d++ = (uint8_t)(((lit >= 15 ? 15 : lit) << 4) | (ml >= 15 ? 15 : ml));
                            if (lit >= 15) d = put_ext(d, lit - 15);
                            copy_lits(d, s.ring, lf >= ring_lo, src, lf, lit);
                            d += lit;
                            d[0] = (uint8_t)off;
                            d[1] = (uint8_t)(off >> 8);
                            d += 2;
                            if (ml >= 15) d = put_ext(d, ml - 15);
                            lf = st + ml + 4;
                        }
                        __syncwarp();
                        if (staged) {
                            const int tot = pend + T, nw = tot >> 2;
                            uint32_t *o32 = d32 + ((op - pend) >> 2);
                            for (int i = lane; i < nw; i += 32) o32[i] = s.stage[i];
                            __syncwarp();
                            if (lane == 0) s.stage[0] = s.stage[nw];
                        } else if (lane == 0 && ((op + T) & 3)) {
                            s.stage[0] = d32[(op + T) >> 2];
                        }
                        op += T;
                        pend = op & 3;
                        anchor = new_anchor;
                        __syncwarp();
                    }
                    entry = __shfl_sync(kFull, X, 31);
                }
                // ---- the prefetched window into the ring
#pragma unroll
                for (int q = 0; q < kW / 128; ++q)
                    s.ring[((w + 2 * kW + 128 * q + 4 * lane) >> 2) & (kRingWords - 1)] = pf[q];
                __syncwarp();
            }
            if (!ovf && pend && lane == 0) d32[(op - pend) >> 2] = s.stage[0];
            __syncwarp();
        }
        if (lane == 0) {
            LzRegion r;
            r.a = a;
            r.first_st = first_st;
            r.first_hdr = first_hdr;
            r.last_end = first_st >= 0 ? anchor : a;
            r.rbytes = ovf ? -1 : op;
            r.ridx = ridx;
            r.pad0 = r.pad1 = 0;
            reg[ri] = r;
        }
        __syncwarp();
    }
}

// Size of each chunk's joined LZ4 block (-1 when a region overflowed).
__global__ void lz4_region_sizes(const LzRegion *reg, const int *in_len, int nchunks, int nreg, int *out_len)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const LzRegion *r = reg + (long long)c * nreg;
    long long lf = 0, size = 0;
    for (int i = 0; i < nreg; ++i) {
        if (r[i].rbytes < 0) {
            out_len[c] = -1;
            return;
        }
        if (r[i].first_st < 0) continue;
        size += 1 + ext_bytes(r[i].first_st - (int)lf) + (r[i].a - lf) + (r[i].rbytes - r[i].first_hdr);
        lf = r[i].last_end;
    }
    const int L = in_len[c];
    size += 1 + ext_bytes(L - (int)lf) + (L - lf);
    out_len[c] = size > 0x7fffffffLL ? -1 : (int)size;
}

// Warp-wide copy of n bytes from src to dst (any alignment); reads up to 4
// bytes past src + n.
__device__ __forceinline__ void wcopy(uint8_t *dst, const uint8_t *src, long long n, int lane)
{
    int h = (int)((4 - (reinterpret_cast<uintptr_t>(dst) & 3)) & 3);
    if (h > n) h = (int)n;
    if (lane < h) dst[lane] = src[lane];
    dst += h;
    src += h;
    n -= h;
    const long long nw = n >> 2;
    const uint32_t sa = (uint32_t)(reinterpret_cast<uintptr_t>(src) & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(src - sa);
    uint32_t *dw = reinterpret_cast<uint32_t *>(dst);
    constexpr int U = 8;
    for (long long i0 = 0; i0 < nw; i0 += 32 * U) {
        uint32_t v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = i0 + 32 * u + lane;
            v[u] = i < nw ? fsr(sw[i], sw[i + 1], 8 * sa) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = i0 + 32 * u + lane;
            if (i < nw) dw[i] = v[u];
        }
    }
    const int t = (int)(n & 3);
    if (lane < t) dst[4 * nw + lane] = src[4 * nw + lane];
}

// Token and literal length bytes of a sequence with `lit` literals; the
// match nibble comes from `mnib`. Returns the bytes written.
__device__ __forceinline__ int put_head(uint8_t *d, int lit, int mnib)
{
    uint8_t *p = d;
    *p++ = (uint8_t)(((lit >= 15 ? 15 : lit) << 4) | mnib);
    if (lit >= 15) p = put_ext(p, lit - 15);
    return (int)(p - d);
}

// One warp per chunk: the joined LZ4 block at out + dst_off[c].
__global__ void __launch_bounds__(256)
lz4_stitch_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks, int nreg,
                  const uint8_t *__restrict__ lz, const long long *lz_off, const LzRegion *reg,
                  uint8_t *__restrict__ out, const long long *dst_off)
{
    const int lane = threadIdx.x & 31;
    const int c = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (c >= nchunks) return;
    const uint8_t *src = in + in_off[c];
    const int L = in_len[c];
    uint8_t *d = out + dst_off[c];
    const LzRegion *r = reg + (long long)c * nreg;
    long long op = 0;
    int lf = 0;
    for (int i = 0; i < nreg; ++i) {
        const LzRegion ri = r[i];
        if (ri.first_st < 0) continue;
        const uint8_t *R = lz + lz_off[c] + area_off(ri.a, ri.ridx);
        const int lit = ri.first_st - lf;
        int hb = 0;
        if (lane == 0) hb = put_head(d + op, lit, R[0] & 15);
        hb = __shfl_sync(kFull, hb, 0);
        op += hb;
        wcopy(d + op, src + lf, ri.a - lf, lane);
        op += ri.a - lf;
        wcopy(d + op, R + ri.first_hdr, ri.rbytes - ri.first_hdr, lane);
        op += ri.rbytes - ri.first_hdr;
        lf = ri.last_end;
    }
    int hb = 0;
    if (lane == 0) hb = put_head(d + op, L - lf, 0);
    hb = __shfl_sync(kFull, hb, 0);
    op += hb;
    wcopy(d + op, src + lf, L - lf, lane);
}

}  // namespace lzr
}  // namespace cz

#ifndef CZ_LZ4REC_NO_LAUNCHERS
using namespace cz;

int cz_lz4rec_smem_bytes(void) { return (int)sizeof(lzr::Smem) * lzr::kWarps; }
int cz_lz4rec_warps_per_cta(void) { return lzr::kWarps; }

long long cz_lz4rec_slot_bytes(long long chunk_max, int bpc)
{
    return ((chunk_max + (chunk_max >> 3) + 64LL * 3 * bpc + 64) + 15) / 16 * 16;
}

cudaError_t cz_launch_lz4_regions(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                  const int *rec_bytes, const long long *blk_dst, long long nblocks, int bpc,
                                  int shuffle, uint8_t *out, const long long *out_off, LzRegion *reg, int grid,
                                  cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    const int smem = cz_lz4rec_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(lzr::lz4_region_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    lzr::lz4_region_kernel<<<grid, lzr::kWarps * 32, smem, st>>>(in, in_off, in_len, nchunks, rec_bytes, blk_dst,
                                                                 nblocks, bpc, shuffle, out, out_off, reg);
    return cudaGetLastError();
}

cudaError_t cz_launch_lz4_region_sizes(const LzRegion *reg, const int *in_len, int nchunks, int bpc, int *out_len,
                                       cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    lzr::lz4_region_sizes<<<(nchunks + 255) / 256, 256, 0, st>>>(reg, in_len, nchunks, 3 * bpc, out_len);
    return cudaGetLastError();
}

cudaError_t cz_launch_lz4_stitch(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks, int bpc,
                                 const uint8_t *lz, const long long *lz_off, const LzRegion *reg, uint8_t *out,
                                 const long long *dst_off, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    const long long threads = (long long)nchunks * 32;
    lzr::lz4_stitch_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(in, in_off, in_len, nchunks, 3 * bpc,
                                                                              lz, lz_off, reg, out, dst_off);
    return cudaGetLastError();
}
#endif
