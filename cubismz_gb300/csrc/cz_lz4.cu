// cz_lz4.cu -- LZ4 legacy block format on the GPU, one warp per chunk.
//
// Encoder: greedy parse, format-compatible with the reference decoder
// LZ4_uncompress_unknownOutputSize (ThirdParty/lz4/lz4.c:802-905): minimum
// match 4, offsets 1..65535, the last 5 bytes are literals and the last
// match starts at least 12 bytes before the end (lz4.c:177-204). A warp
// takes super-windows of 512 or 768 positions (see window_for):
//   * probe  -- 4 positions per lane per step from coalesced word loads; a
//     hash table of 1024 entries per warp in shared memory holds position
//     (mod 2^18) and a 14-bit tag of the 4-byte sequence, so most false
//     candidates are dropped without reading memory;
//   * walk   -- lane k parses its 16 or 24 positions greedily, jumping
//     from one position with a candidate to the next (a bitmask of its
//     candidate slots) and measuring matches against memory;
//   * merge  -- lane k keeps the sequences that start at or after the end
//     of the last kept match of lanes < k (one ballot when no match crosses
//     a later lane's last start, the exact serial rule otherwise);
//   * emit   -- a warp scan places every kept sequence, each lane writes its
//     own; literal runs over 32 bytes are copied by the whole warp.
// Parse effort (a template level, cz_set_lz4_effort): 1 (default) extends
// kept matches backwards over equal bytes (lz4.c's "catch up") and keeps
// the tail of a match that a lower lane's match overlaps; 2 also takes
// repeats at distance 1-3 that the table misses and starts each lane's
// walk 8 positions early; 0 does neither.
// Windows without a match advance faster after repeated misses (the
// reference's acceleration idea, lz4.c:389-393). Chunks of block records
// ([int32 nbytes][mask][4 byte planes], shuffle on) skip the search over
// byte planes 1 and 2 -- the two middle mantissa bytes, which do not
// compress -- and copy them as literals; those literal bytes are not even
// copied here: the encoder leaves their span of its output unwritten and
// records it per chunk, and the gather that packs the stream copies them
// straight from the records. The same parse in SEQ mode feeds the DEFLATE
// encoder (cz_zlib.cu).
// Decoder: the same acceptance tests and error convention as
// LZ4_uncompress_unknownOutputSize (-(input position) on malformed input; an
// empty input yields 0). Windows of 128 input bytes are parsed
// speculatively (every lane decodes tokens at 4 candidate positions; jump
// tables by pointer doubling find the real sequences), output is staged in a
// 4 KB per-warp ring and flushed with word stores; overlapping matches
// repeat their first `offset` bytes, the byte-serial copy semantics. Short
// matches are copied by their own lanes in rounds (sources before the
// window first, then those whose sources the earlier rounds completed);
// long ones by the whole warp. For one-record chunks of shuffled records a
// literal run that covers byte planes 1 and 2 whole stays in the input
// (hole), where later matches and the decode kernel read it.
#include "cz_codec.h"
#include "cz_deflate.cuh"

namespace cz {

constexpr int kHashLog = 10;
constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kMinMatch = 4, kLastLiterals = 5, kMfLimit = 12;

__device__ __forceinline__ uint32_t lz_hash(uint32_t v) { return (v * 2654435761u) >> (32 - kHashLog); }

__device__ __forceinline__ unsigned lanemask_lt_()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// 32-bit little-endian word at any byte address (two aligned loads).
__device__ __forceinline__ uint32_t rd32u(const uint8_t *p)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    return sh ? __funnelshift_r(w[0], w[1], sh) : w[0];
}

// 16 bytes at any byte address as four little-endian words: five aligned
// loads, all issued before any use. May read up to 19 bytes past p (inputs
// carry tail room).
__device__ __forceinline__ void rd16u(const uint8_t *p, uint32_t (&v)[4])
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    uint32_t x[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) x[j] = w[j];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = sh ? __funnelshift_r(x[j], x[j + 1], sh) : x[j];
}

// Warp-wide copy of n bytes; 4-byte stores once dst is aligned. May read up
// to 4 bytes past src+n (inputs carry tail room).
__device__ __forceinline__ void warp_copy(uint8_t *dst, const uint8_t *src, int n, int lane)
{
    int h = (int)((4 - (reinterpret_cast<uintptr_t>(dst) & 3)) & 3);
    if (h > n) h = n;
    if (lane < h) dst[lane] = src[lane];
    dst += h;
    src += h;
    n -= h;
    const int nw = n >> 2;
    const uint32_t sa = (uint32_t)(reinterpret_cast<uintptr_t>(src) & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(src - sa);
    uint32_t *dw = reinterpret_cast<uint32_t *>(dst);
    // 8 words per lane in flight: every load of a round before its stores
    constexpr int U = 8;
    for (int i0 = 0; i0 < nw; i0 += 32 * U) {
        uint32_t v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + 32 * u + lane;
            v[u] = i < nw ? (sa ? __funnelshift_r(sw[i], sw[i + 1], 8 * sa) : sw[i]) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + 32 * u + lane;
            if (i < nw) dw[i] = v[u];
        }
    }
    const int t = n & 3;
    if (lane < t) dst[4 * nw + lane] = src[4 * nw + lane];
}

// n <= 32 bytes, 4 per step, so that the cost follows n (most literal runs
// between matches are 0-4 bytes). Source and destination never overlap. May
// read up to 7 bytes past s + n (inputs carry tail room).
__device__ __forceinline__ void copy_short(uint8_t *__restrict__ d, const uint8_t *__restrict__ s, int n)
{
    for (int i = 0; i < n; i += 4) {
        const uint32_t w = rd32u(s + i);
        d[i] = (uint8_t)w;
        if (i + 1 < n) d[i + 1] = (uint8_t)(w >> 8);
        if (i + 2 < n) d[i + 2] = (uint8_t)(w >> 16);
        if (i + 3 < n) d[i + 3] = (uint8_t)(w >> 24);
    }
}

// Bytes of a length field's continuation: n/255 bytes of 255, then n%255.
__device__ __forceinline__ int len_bytes(int n) { return n / 255 + 1; }
__device__ __forceinline__ void put_len_serial(uint8_t *d, int n)
{
    for (; n >= 255; n -= 255) *d++ = 255;
    *d = (uint8_t)n;
}

// Record layout of a chunk: literal-only range [lo, hi) of the current
// record (its byte planes 1 and 2) and where the next record starts.
struct Skip {
    int lo, hi, next;
    bool on;
};
__device__ __forceinline__ void next_skip(Skip &k, const uint8_t *src, int L)
{
    while (k.on) {
        if (k.next + 4 > L) break;
        const int nb = (int)rd32u(src + k.next);
        if (nb < 4096 || nb > 4096 + 4 * 32768 || k.next + 4 + nb > L) break;
        const int S = (nb - 4096) / 4;
        k.lo = k.next + 4 + 4096 + S;
        k.hi = k.lo + 2 * S;
        k.next += 4 + nb;
        if (k.hi > k.lo) return;
    }
    k.on = false;
    k.lo = k.hi = L + 1;
}

// ------------------------------------------------------------------ encode
// Per warp, per super-window of kSW positions:
//   probe  -- 128 positions per step (4 per lane): hash, table lookup and
//             insert, verification against the stored 4-byte sequence;
//             the candidate offset per position goes to info[] (0: none);
//   walk   -- lane k walks positions [base+32k, base+32k+32) greedily
//             (take the match at the cursor, measure it, jump past it,
//             else step 1);
//   merge  -- lane k keeps its sequences that start at or after the end of
//             the last kept match of lanes < k: the kept matches never
//             overlap, so the parse stays valid LZ4 without any lane
//             waiting for another;
//   emit   -- every lane sizes its kept sequences, a warp scan places them,
//             every lane writes its own; literal runs longer than 32 bytes
//             are queued and copied by the whole warp.
constexpr int kOvl = 8;
// super-window sizes: 768 positions when every chunk of the launch is
// resident at once (fewer windows per chunk), 512 otherwise (a smaller
// per-warp footprint, so more chunks share an SM)
constexpr int kWinSmall = 512, kWinLarge = 768;
constexpr int kMinHole = 256;  // smallest literal-only span left to the gather
// Hash table entry: position modulo 2^18 in the high bits, a 14-bit tag of
// the 4-byte sequence in the low bits. A tag hit is only a candidate: the
// walk measures the match from its first byte and drops it below 4 bytes.
constexpr uint32_t kPosMask = (1u << 18) - 1;
__device__ __forceinline__ uint32_t lz_tag(uint32_t v) { return (v * 0x85ebca77u) >> 18; }

// 8 bytes at any byte address as two little-endian words (three aligned
// loads). May read up to 11 bytes past p.
__device__ __forceinline__ void rd8u(const uint8_t *p, uint32_t (&v)[2])
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    const uint32_t x0 = w[0], x1 = w[1], x2 = w[2];
    v[0] = sh ? __funnelshift_r(x0, x1, sh) : x0;
    v[1] = sh ? __funnelshift_r(x1, x2, sh) : x1;
}

// exact match length from (p, cand), starting `known` bytes in (lane-local):
// the first 8 bytes on their own (most matches are 4-8 bytes long), then 16
// bytes per round trip to memory
__device__ __forceinline__ int match_len(const uint8_t *src, int p, int cand, int known, int matchlimit)
{
    int len = known;
    {
        uint32_t a[2], b[2];
        rd8u(src + p + len, a);
        rd8u(src + cand + len, b);
        const uint32_t x0 = a[0] ^ b[0], x1 = a[1] ^ b[1];
        const int k = x0 ? (__ffs(x0) - 1) >> 3 : x1 ? 4 + ((__ffs(x1) - 1) >> 3) : 8;
        len += k;
        if (k < 8) return len < matchlimit - p ? len : matchlimit - p;
    }
    while (p + len < matchlimit) {
        uint32_t a[4], b[4];
        rd16u(src + p + len, a);
        rd16u(src + cand + len, b);
        int k = 16;
#pragma unroll
        for (int j = 3; j >= 0; --j) {
            const uint32_t x = a[j] ^ b[j];
            if (x) k = 4 * j + ((__ffs(x) - 1) >> 3);
        }
        len += k;
        if (k < 16) break;
    }
    return len < matchlimit - p ? len : matchlimit - p;
}

// match_len from byte 0, and how many of the (at most 4) bytes before p
// equal the bytes before cand (0 when cand < 4): the words before both
// positions are loaded with the first 8 bytes, so the count costs no
// extra round trip to memory.
__device__ __forceinline__ int match_len_back(const uint8_t *src, int p, int cand, int matchlimit, int &back)
{
    const uintptr_t pa = reinterpret_cast<uintptr_t>(src + p), ca = reinterpret_cast<uintptr_t>(src + cand);
    const uint32_t *pw = reinterpret_cast<const uint32_t *>(pa & ~(uintptr_t)3);
    const uint32_t *cw = reinterpret_cast<const uint32_t *>(ca & ~(uintptr_t)3);
    const uint32_t ps = (uint32_t)(pa & 3) * 8, cs = (uint32_t)(ca & 3) * 8;
    const bool before = cand >= 4;  // then p > cand >= 4 too: both words lie inside the chunk
    const uint32_t p0 = pw[0], p1 = pw[1], p2 = pw[2], pm = before ? pw[-1] : 0u;
    const uint32_t c0 = cw[0], c1 = cw[1], c2 = cw[2], cm = before ? cw[-1] : 0u;
    const uint32_t a0 = ps ? __funnelshift_r(p0, p1, ps) : p0, a1 = ps ? __funnelshift_r(p1, p2, ps) : p1;
    const uint32_t b0 = cs ? __funnelshift_r(c0, c1, cs) : c0, b1 = cs ? __funnelshift_r(c1, c2, cs) : c1;
    const uint32_t ab = ps ? __funnelshift_r(pm, p0, ps) : pm, bb = cs ? __funnelshift_r(cm, c0, cs) : cm;
    back = before ? __clz(ab ^ bb) >> 3 : 0;
    const uint32_t x0 = a0 ^ b0, x1 = a1 ^ b1;
    const int k = x0 ? (__ffs(x0) - 1) >> 3 : x1 ? 4 + ((__ffs(x1) - 1) >> 3) : 8;
    if (k < 8) return k < matchlimit - p ? k : matchlimit - p;
    return match_len(src, p, cand, 8, matchlimit);
}

// SEQ: the parse for the DEFLATE encoder instead of LZ4 bytes -- distances up
// to 32 KiB, and per kept sequence one 8-byte record (literal run, match
// length, distance; zl::seq_pack) at out + out_off[c]; the last record holds
// the tail literals. out_len[c] = record bytes, -1 past the capacity.
// Shared memory of one encoder warp for super-windows of SW positions.
template <int SW>
struct LzEncWarp {
    uint32_t table[1 << kHashLog];
    int4 longq[32];                   // (dst offset, src offset, n, -)
    uint32_t seq[32][SW / 128];       // start - base | back extension << 12 | offset << 16
    int lens[32][SW / 128];
    uint16_t info[SW];                // candidate offset per position, 0: none
    int nlong;
};

template <int kLzWarps, bool SEQ, int kEffort, int kSW>
__global__ void __launch_bounds__(kLzWarps * 32)
lz4_encode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, int *out_len, int records, int4 *hole)
{
    constexpr int kSub = kSW / 32, kMaxSeqLane = kSub / 4;  // positions and sequences per lane
    using LzEncWarp = cz::LzEncWarp<kSW>;
    constexpr bool kThorough = kEffort >= 2;
    constexpr int kMaxOff = SEQ ? zl::kMaxDist : 65535;
    // up to 8 warps in static shared memory; 16 in dynamic
    extern __shared__ __align__(16) unsigned char lz_enc_smem[];
    __shared__ LzEncWarp lz_enc_static[kLzWarps <= 8 ? kLzWarps : 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    LzEncWarp &ws = (kLzWarps <= 8 ? lz_enc_static : reinterpret_cast<LzEncWarp *>(lz_enc_smem))[wib];
    uint32_t *table = ws.table;
    uint16_t *info = ws.info;
    uint32_t *myseq = ws.seq[lane];
    int *mylen = ws.lens[lane];
    int4 *longq = ws.longq;
    int &nlong = ws.nlong;
    const int gw = blockIdx.x * kLzWarps + wib, nw = gridDim.x * kLzWarps;

    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int L = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int cap = SEQ ? 8 * (L / 4 + 2) : L + L / 255 + 16;
        for (int i = lane; i < (1 << kHashLog); i += 32) table[i] = kEmpty;
        __syncwarp();
        int pos = 0, anchor = 0, op = 0, miss = 0;
        bool overflow = false;
        // the literal-only planes last jumped over, and whether the chunk's
        // one deferred copy (left to the gather) is taken
        int hlo = 0, hhi = 0;
        bool deferred = hole == nullptr || !records;
        if (hole && lane == 0) hole[c] = make_int4(0, 0, 0, 0);  // written for every chunk
        Skip sk;
        sk.on = records != 0;
        sk.next = 0;
        sk.lo = sk.hi = L + 1;
        if (sk.on) next_skip(sk, src, L);
        const int mflimit = L - kMfLimit, matchlimit = L - kLastLiterals;
        while (L >= kMfLimit + 1 && pos <= mflimit && !overflow) {
            if (pos >= sk.lo) {  // literal-only planes: jump over them
                if (pos < sk.hi) pos = sk.hi;
                hlo = sk.lo;
                hhi = sk.hi;
                next_skip(sk, src, L);
                miss = 0;
                continue;
            }
            const int base = pos;
            int end = base + kSW;
            if (end > mflimit + 1) end = mflimit + 1;
            if (end > sk.lo) end = sk.lo;
            // ---- probe [base, end): the window's words are loaded up front
            // and the next window is prefetched into L1
            bool any_match = false;
            constexpr int kSteps = (kSW + 4 + 127) / 128;
            uint32_t wv[kSteps], wx[kSteps];
            // effort 2: the word before the window (for the distance 1-3
            // candidates of its first positions)
            uint32_t wprev = kThorough && (base & ~3) >= 4
                                 ? __ldg(reinterpret_cast<const uint32_t *>(src + (base & ~3) - 4))
                                 : 0u;
#pragma unroll
            for (int k = 0; k < kSteps; ++k) {
                const int wpos = (base & ~3) + 128 * k + 4 * lane;
                wv[k] = wpos + 4 <= L ? __ldg(reinterpret_cast<const uint32_t *>(src + wpos)) : 0u;
                wx[k] = lane == 31 && wpos + 8 <= L ? __ldg(reinterpret_cast<const uint32_t *>(src + wpos + 4)) : 0u;
            }
            if (lane < kSteps && (base & ~3) + kSW + 128 * lane < L)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(src + (base & ~3) + kSW + 128 * lane));
#pragma unroll
            for (int k = 0; k < kSteps; ++k) {
                const int wb = (base & ~3) + 128 * k;
                if (wb >= end) break;
                const int wpos = wb + 4 * lane;
                const uint32_t w0 = wv[k];
                uint32_t w1 = __shfl_down_sync(0xffffffffu, w0, 1);
                if (lane == 31) w1 = wx[k];
                // sx[3 + i]: the 4-byte sequence at wpos + i, i = -3..3
                // (i < 0 only with effort 2)
                uint32_t sx[7], h[4];
                bool valid[4];
                if (kThorough) {
                    uint32_t wp = __shfl_up_sync(0xffffffffu, w0, 1);
                    if (lane == 0) wp = wprev;
                    wprev = __shfl_sync(0xffffffffu, w0, 31);
#pragma unroll
                    for (int i = 0; i < 3; ++i) sx[i] = __funnelshift_r(wp, w0, 8 + 8 * i);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = wpos + j;
                    valid[j] = p >= base && p < end;
                    sx[3 + j] = j ? __funnelshift_r(w0, w1, 8 * j) : w0;
                    h[j] = lz_hash(sx[3 + j]);
                }
                const uint32_t *seq = sx + 3;
                uint32_t e[4], tag[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    e[j] = table[h[j]];
                    tag[j] = lz_tag(seq[j]);
                }
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (valid[j]) table[h[j]] = (((uint32_t)(wpos + j) & kPosMask) << 14) | tag[j];
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = wpos + j;
                    const int off = (int)(((uint32_t)p - (e[j] >> 14)) & kPosMask);
                    int v = 0;
                    if (valid[j] && e[j] != kEmpty && (e[j] & 0x3fff) == tag[j] && off >= 1 && off <= kMaxOff && off <= p)
                        v = off;  // the walk verifies and measures chosen candidates
                    if (kThorough) {
                        // the table is read before this step's positions
                        // enter it, so a repeat at distance 1-3 (runs, short
                        // periods) is taken from the sequences directly
                        const int near = seq[j] == sx[2 + j] ? 1 : seq[j] == sx[1 + j] ? 2 : seq[j] == sx[j] ? 3 : 0;
                        if (near && p >= near) v = near;
                    }
                    if (valid[j]) info[p - base] = (uint16_t)v;
                    any_match |= v != 0;
                }
            }
            __syncwarp();
            if (!__any_sync(0xffffffffu, any_match)) {
                ++miss;
                pos = end + (miss > 2 ? (miss - 2) * 256 : 0);
                continue;
            }
            miss = 0;
            // ---- walk: lane-local greedy parse of [base + kSub*lane, +kSub)
            // (effort 2: entered kOvl positions early, at the end of the
            // lower lane's segment, so that it mostly lands on the serial
            // parse's path); a kept match also records how many bytes before
            // it equal the bytes before its source (at most 4), taken into
            // the match in the emission as far as the literal run allows
            // (effort >= 1: lz4.c's backward "catch up", lz4.c:586-587)
            int ns = 0, last_start = -1, last_end = -1;
            {
                const int w0p = base + kSub * lane;
                const int qe = min(w0p + kSub, end);
                const int qs = kThorough && lane ? w0p - kOvl : w0p;
                // the walk's positions that have a candidate (bit i: qs + i),
                // so that it jumps over literal positions
                constexpr int kNq = kThorough ? kSub + kOvl : kSub;
                uint32_t cm = 0;
                if (qe > qs) {
                    const uint4 *iv = reinterpret_cast<const uint4 *>(info + (qs - base));  // 16-byte aligned
#pragma unroll
                    for (int v = 0; v < kNq / 8; ++v) {
                        const uint4 a = iv[v];
                        const uint32_t iw[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            cm |= (uint32_t)((iw[i] & 0xffffu) != 0) << (8 * v + 2 * i) |
                                  (uint32_t)((iw[i] >> 16) != 0) << (8 * v + 2 * i + 1);
                    }
                    if (qe - qs < kNq) cm &= (1u << (qe - qs)) - 1u;
                }
                int q = qs;
                while (q < qe) {
                    const uint32_t m = cm >> (q - qs);
                    if (!m) break;
                    q += __ffs(m) - 1;
                    const int off = info[q - base];
                    int ext = 0;
                    const int len = !off ? 0
                                    : kEffort >= 1 ? match_len_back(src, q, q - off, matchlimit, ext)
                                                   : match_len(src, q, q - off, 0, matchlimit);
                    if (len >= kMinMatch) {
                        if (q >= w0p) {
                            myseq[ns] = (uint32_t)(q - base) | (uint32_t)ext << 12 | (uint32_t)off << 16;
                            mylen[ns] = len;
                            ++ns;
                            last_start = q;
                            last_end = q + len;
                        }
                        q += len;
                    } else {
                        ++q;
                    }
                }
            }
            // ---- merge: P_k = end of the last kept match of lanes < k. With
            // effort >= 1 a match [s, e) that starts before the literal
            // position P is kept from P on when that part is still a match
            // (>= 4 bytes) that may follow a literal run (P <= mflimit).
            auto survives = [&](int s, int e, int P) {
                return s >= P || (kEffort >= 1 && e - P >= kMinMatch && P <= mflimit);
            };
            // Usually every lane keeps its last sequence, so P_k is the end
            // of the nearest lower lane's last match; where a match reaches
            // past a later lane's last start, the exact serial rule runs.
            const unsigned has = __ballot_sync(0xffffffffu, ns > 0);
            const unsigned lower = has & lanemask_lt_();
            int myP = __shfl_sync(0xffffffffu, last_end, lower ? 31 - __clz(lower) : 0);
            if (!lower) myP = anchor;
            int P = has ? __shfl_sync(0xffffffffu, last_end, 31 - __clz(has)) : anchor;
            const unsigned bad = __ballot_sync(0xffffffffu, ns > 0 && !survives(last_start, last_end, myP));
            if (bad) {
                // lanes below the first failing one are exact; from there the
                // serial rule over the lanes that have sequences
                const int f = __ffs(bad) - 1;
                P = __shfl_sync(0xffffffffu, myP, f);
                for (unsigned rest = has & ~((1u << f) - 1u); rest; rest &= rest - 1u) {
                    const int k = __ffs(rest) - 1;
                    const int ls = __shfl_sync(0xffffffffu, last_start, k);
                    const int le = __shfl_sync(0xffffffffu, last_end, k);
                    if (lane == k) myP = P;
                    if (survives(ls, le, P)) P = le;
                }
            }
            // ---- emit: kept sequences are those starting at or after myP
            int lit_from = myP, bytes = 0, nkeep = 0;
            for (int i = 0; i < ns; ++i) {
                const int s0 = base + (int)(myseq[i] & 0xfff);
                if (!survives(s0, s0 + mylen[i], lit_from)) continue;
                const int st = max(s0 - (int)((myseq[i] >> 12) & 7), lit_from);
                const int l = st - lit_from, ml = s0 + mylen[i] - st - kMinMatch;
                bytes += SEQ ? 8 : 1 + (l >= 15 ? len_bytes(l - 15) : 0) + l + 2 + (ml >= 15 ? len_bytes(ml - 15) : 0);
                lit_from = s0 + mylen[i];
                ++nkeep;
            }
            int incl = bytes;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if ((long long)op + total + 1 + kLastLiterals > cap) {
                overflow = true;
                break;
            }
            if (lane == 0) nlong = 0;
            __syncwarp();
            if (SEQ) {
                int at = op + incl - bytes;
                lit_from = myP;
                for (int i = 0; i < ns; ++i) {
                    const int s0 = base + (int)(myseq[i] & 0xfff);
                    if (!survives(s0, s0 + mylen[i], lit_from)) continue;
                    const int st = max(s0 - (int)((myseq[i] >> 12) & 7), lit_from);
                    *reinterpret_cast<unsigned long long *>(dst + at) =
                        zl::seq_pack(st - lit_from, s0 + mylen[i] - st, (int)(myseq[i] >> 16));
                    at += 8;
                    lit_from = s0 + mylen[i];
                }
            } else {
                int at = op + incl - bytes;
                lit_from = myP;
                for (int i = 0; i < ns; ++i) {
                    const int s0 = base + (int)(myseq[i] & 0xfff);
                    if (!survives(s0, s0 + mylen[i], lit_from)) continue;
                    const int st = max(s0 - (int)((myseq[i] >> 12) & 7), lit_from);
                    const int l = st - lit_from, ml = s0 + mylen[i] - st - kMinMatch, off = (int)(myseq[i] >> 16);
                    uint8_t *d = dst + at;
                    *d++ = (uint8_t)(((l >= 15 ? 15 : l) << 4) | (ml >= 15 ? 15 : ml));
                    if (l >= 15) {
                        put_len_serial(d, l - 15);
                        d += len_bytes(l - 15);
                    }
                    if (l <= 32) {
                        copy_short(d, src + lit_from, l);
                    } else {
                        const int slot = atomicAdd(&nlong, 1);
                        if (slot < 32) longq[slot] = make_int4((int)(d - dst), lit_from, l, 0);
                    }
                    d += l;
                    d[0] = (uint8_t)off;
                    d[1] = (uint8_t)(off >> 8);
                    if (ml >= 15) put_len_serial(d + 2, ml - 15);
                    at += 1 + (l >= 15 ? len_bytes(l - 15) : 0) + l + 2 + (ml >= 15 ? len_bytes(ml - 15) : 0);
                    lit_from = s0 + mylen[i];
                }
            }
            __syncwarp();
            const int nl = nlong;
            if (nl > 32) {  // cannot happen: a long run (> 32 bytes) only before a lane's first sequence
                overflow = true;
                break;
            }
            for (int i = 0; i < nl; ++i) {
                const int4 t = longq[i];
                // the planes inside this run go to the gather (once per
                // chunk): it copies them from the records into the stream
                const int a = max(t.y, hlo), b = min(t.y + t.z, hhi);
                if (!deferred && b - a >= kMinHole) {
                    warp_copy(dst + t.x, src + t.y, a - t.y, lane);
                    warp_copy(dst + t.x + (b - t.y), src + b, t.y + t.z - b, lane);
                    if (lane == 0) hole[c] = make_int4(t.x + (a - t.y), a, b - a, 0);
                    deferred = true;
                } else {
                    warp_copy(dst + t.x, src + t.y, t.z, lane);
                }
            }
            __syncwarp();
            op += total;
            anchor = P;
            pos = end > P ? end : P;
        }
        if (!overflow && SEQ) {
            if (op + 8 > cap) {
                overflow = true;
            } else {
                if (lane == 0) *reinterpret_cast<unsigned long long *>(dst + op) = zl::seq_pack(L - anchor, 0, 0);
                op += 8;
            }
        } else if (!overflow) {
            const int lit = L - anchor;
            const int need = 1 + (lit >= 15 ? len_bytes(lit - 15) : 0) + lit;
            if (op + need > cap) {
                overflow = true;
            } else {
                if (lane == 0) {
                    dst[op] = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
                    if (lit >= 15) put_len_serial(dst + op + 1, lit - 15);
                }
                op += 1 + (lit >= 15 ? len_bytes(lit - 15) : 0);
                const int a = max(anchor, hlo), b = min(L, hhi);
                if (!deferred && b - a >= kMinHole) {  // the planes to the gather, as above
                    warp_copy(dst + op, src + anchor, a - anchor, lane);
                    warp_copy(dst + op + (b - anchor), src + b, L - b, lane);
                    if (lane == 0) hole[c] = make_int4(op + (a - anchor), a, b - a, 0);
                    deferred = true;
                } else {
                    warp_copy(dst + op, src + anchor, lit, lane);
                }
                op += lit;
            }
        }
        if (lane == 0) out_len[c] = overflow ? -1 : op;
        __syncwarp();
    }
}

// ------------------------------------------------------------------ decode
// Length continuation bytes from ip while they are 255 and ip < lim;
// returns their sum and leaves ip after the last byte read.
__device__ __forceinline__ long long get_len(const uint8_t *src, int &ip, int lim)
{
    long long sum = 0;
    while (ip < lim) {
        const int s = src[ip++];
        sum += s;
        if (s != 255) break;
    }
    return sum;
}

// Parallel parse. The decoder reads a window of kWin input bytes starting
// at the current sequence. Every lane decodes the token at 4 candidate
// positions as if a sequence started there (literal length, offset, match
// length, position of the next token); only the candidates reachable from
// the window's first position are real sequences. Jump tables T_b (2^b
// steps along the next-token chain, built by pointer doubling in shared
// memory) let lane k find the k-th sequence directly. Candidates whose
// length fields run longer than kFastExt continuation bytes are flagged
// and decoded serially when the chain reaches them.
constexpr int kWin = 128, kFastExt = 8, kExit = kWin;
// Output ring per warp: the last kRing bytes of output. A window adds at
// most kStage bytes, so at least kRing - kStage bytes of history stay
// readable while it is written (about 99% of match sources in block-record
// chunks lie within 3 KB).
constexpr int kRing = 4096, kMask = kRing - 1, kStage = 1024;
constexpr int kTermIn = 1 << 16, kSlow = 1 << 17;  // flags above the 16-bit offset

// Continuation bytes like get_len, at most kFastExt of them: false if the
// field is longer (the caller then decodes the sequence serially).
__device__ __forceinline__ bool get_len_fast(const uint8_t *src, int &ip, int lim, int &sum)
{
#pragma unroll 1
    for (int k = 0; k < kFastExt; ++k) {
        if (ip >= lim) return true;
        const int s = __ldg(src + ip++);
        sum += s;
        if (s != 255) return true;
    }
    return ip >= lim;
}

// n <= 8 bytes from read-only input into the ring at output position o;
// all loads before the stores.
__device__ __forceinline__ void copy_lit(uint8_t *ring, int o, const uint8_t *s, int n)
{
    uint8_t b[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) b[j] = j < n ? __ldg(s + j) : (uint8_t)0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < n) ring[(o + j) & kMask] = b[j];
}

// Byte k of a match at output ms comes from ms - off + (k mod off): the
// byte-serial copy repeats the first `off` bytes when off < length.
__device__ __forceinline__ int msrc(int k, int off, int ml) { return off >= ml ? k : k % off; }

// Byte planes 1 and 2 of a record chunk that the decoder left in its input
// (a literal run it did not copy): output [out, out + len) is input
// [in, in + len); len 0: none.
struct LzHole {
    int out = 0, len = 0, in = 0;
};

// Output byte x from global memory: from the input inside the hole, else
// from the output (via L2).
__device__ __forceinline__ uint8_t old_byte(const uint8_t *src, const uint8_t *dst, const LzHole &h, int x)
{
    return (unsigned)(x - h.out) < (unsigned)h.len ? __ldg(src + h.in + (x - h.out)) : __ldcg(dst + x);
}

// Output byte x, x < the window's start: from the ring when it is still
// held there (x >= lo), else from global memory.
__device__ __forceinline__ uint8_t out_byte(const uint8_t *ring, const uint8_t *src, const uint8_t *dst,
                                            const LzHole &h, int x, int lo)
{
    return x >= lo ? ring[x & kMask] : old_byte(src, dst, h, x);
}

// ml <= 8 bytes of a match at ms whose sources lie before the window and
// in the ring; r runs through the source positions modulo off.
__device__ __forceinline__ void copy_match(uint8_t *ring, int ms, int off, int ml)
{
    uint8_t b[8];
    int r = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        b[j] = j < ml ? ring[(ms - off + r) & kMask] : (uint8_t)0;
        r = r + 1 == off ? 0 : r + 1;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < ml) ring[(ms + j) & kMask] = b[j];
}

// ml <= 8 bytes of a match at ms whose sources all lie before lo (in global
// memory, or in the input where the hole is); r as in copy_match.
__device__ __forceinline__ void copy_match_old(uint8_t *ring, int ms, int off, int ml, const uint8_t *src,
                                               const uint8_t *dst, const LzHole &h)
{
    uint8_t b[8];
    int r = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        b[j] = j < ml ? old_byte(src, dst, h, ms - off + r) : (uint8_t)0;
        r = r + 1 == off ? 0 : r + 1;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < ml) ring[(ms + j) & kMask] = b[j];
}

// n bytes of the ring starting at ring offset r (r + n <= kRing) to d (any
// alignment): 4-byte stores once d is aligned.
__device__ __forceinline__ void flush(uint8_t *d, const uint8_t *ring, int r, int n, int lane)
{
    int h = (int)((4 - (reinterpret_cast<uintptr_t>(d) & 3)) & 3);
    if (h > n) h = n;
    if (lane < h) d[lane] = ring[r + lane];
    const int nw = (n - h) >> 2, b = r + h, sh = 8 * (b & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(ring) + (b >> 2);
    uint32_t *dw = reinterpret_cast<uint32_t *>(d + h);
    for (int i = lane; i < nw; i += 32) dw[i] = sh ? __funnelshift_r(sw[i], sw[i + 1], sh) : sw[i];
    const int t = (n - h) & 3;
    if (lane < t) d[h + 4 * nw + lane] = ring[b + 4 * nw + lane];
}

__global__ void __launch_bounds__(128)
lz4_decode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, const int *out_cap, int *out_len,
                  int4 *hole)
{
    __shared__ int4 cand_all[4][kWin];           // (literal start, literal length, match length, flags)
    __shared__ int next_all[4][kWin];            // input position after the candidate's sequence
    __shared__ __align__(16) uint8_t jump_all[4][5][kWin + 4];  // T_b; kExit: leaves the window
    __shared__ __align__(16) uint8_t ring_all[4][kRing + 16];  // recent output (16 bytes of slack)
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int4 *cand = cand_all[wib];
    int *nextp = next_all[wib];
    uint8_t(*T)[kWin + 4] = jump_all[wib];
    uint8_t *ring = ring_all[wib];
    if (lane < 4) {
#pragma unroll
        for (int b = 0; b < 5; ++b) T[b][kWin + lane] = (uint8_t)kExit;
    }
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int iend = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int oend = out_cap[c];
        int s0 = 0, op = 0, err = 0, ring_lo = 0;  // output before ring_lo is not in the ring
        bool done = false;
        LzHole hl;
        if (hole && lane == 0) hole[c] = make_int4(0, 0, 0, 0);  // written for every chunk
        // a literal run of n bytes from input i to output o, except the
        // record's byte planes 1 and 2 when it covers them whole (hole
        // given, record chunks: the record's byte count is output bytes 0-3)
        auto lit_run = [&](int o, int i, int n) {
            int a = 0, b = 0;
            if (hole && hl.len == 0 && o >= 4) {
                const int nb = (int)__ldcg(dst) | (int)__ldcg(dst + 1) << 8 | (int)__ldcg(dst + 2) << 16 |
                               (int)__ldcg(dst + 3) << 24;
                if (nb >= 4096 && nb <= 4096 + 4 * 32768 && ((nb - 4096) & 3) == 0) {
                    const int S = (nb - 4096) >> 2;
                    a = 4 + 4096 + S;
                    b = a + 2 * S;
                    if (!(o <= a && o + n >= b && b - a >= kMinHole)) a = b = 0;
                }
            }
            if (b > a) {
                warp_copy(dst + o, src + i, a - o, lane);
                warp_copy(dst + b, src + i + (b - o), o + n - b, lane);
                hl.out = a;
                hl.len = b - a;
                hl.in = i + (a - o);
                if (lane == 0) hole[c] = make_int4(hl.out, hl.in, hl.len, 0);
            } else {
                warp_copy(dst + o, src + i, n, lane);
            }
        };
        if (iend <= 0) {
            if (lane == 0) out_len[c] = 0;  // lz4.c:836: error exit at position 0
            continue;
        }
        while (!done && !err) {
            // ---- candidates s0 + 4*lane + j; the next window's input into L1
            if (lane < 2 && s0 + kWin + 128 * lane < iend)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(src + s0 + kWin + 128 * lane));
            {  // phase-major over the 4 candidates, so that their loads overlap
                int tok[4], ip[4], lit[4], ml[4], nx[4];
                bool more[4], stat[4];  // stat: a plain sequence so far
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = s0 + 4 * lane + j;
                    tok[j] = p < iend ? (int)__ldg(src + p) : -1;
                    ip[j] = p + 1;
                    lit[j] = (tok[j] >> 4) & 15;
                    ml[j] = tok[j] & 15;
                    nx[j] = 0;
                }
                // literal length continuation (lz4.c:846-850): the first byte
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    more[j] = false;
                    if (tok[j] >= 0 && lit[j] == 15 && ip[j] < iend) {
                        const int e = __ldg(src + ip[j]);
                        ++ip[j];
                        lit[j] += e;
                        more[j] = e == 255;
                    }
                }
                // ... and the rare longer ones
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    stat[j] = tok[j] >= 0;
                    if (more[j]) stat[j] = get_len_fast(src, ip[j], iend, lit[j]);
                }
                int flags[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    flags[j] = 0;
                    if (tok[j] >= 0) {
                        if (!stat[j]) flags[j] = kSlow;
                        else if (lit[j] > iend - ip[j] - (2 + 1 + kLastLiterals)) flags[j] = kTermIn;  // lz4.c:851
                    }
                    stat[j] = tok[j] >= 0 && flags[j] == 0;
                    if (stat[j]) nx[j] = ip[j] + lit[j] + 2;  // the offset is read for real sequences only
                }
                // match length continuation (lz4.c:873-882)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    more[j] = false;
                    if (stat[j] && ml[j] == 15 && nx[j] < iend - (kLastLiterals + 1)) {
                        const int e = __ldg(src + nx[j]);
                        ++nx[j];
                        ml[j] += e;
                        more[j] = e == 255;
                    }
                }
                uint32_t tword = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (more[j] && !get_len_fast(src, nx[j], iend - (kLastLiterals + 1), ml[j])) flags[j] = kSlow;
                    ml[j] += kMinMatch;
                    int t = kExit;
                    if (stat[j] && flags[j] == 0 && nx[j] - s0 < kWin) t = nx[j] - s0;
                    if (flags[j]) nx[j] = 0;
                    cand[4 * lane + j] = make_int4(ip[j], lit[j], ml[j], flags[j]);
                    nextp[4 * lane + j] = nx[j];
                    tword |= (uint32_t)t << (8 * j);
                }
                reinterpret_cast<uint32_t *>(T[0])[lane] = tword;
            }
            __syncwarp();
#pragma unroll
            for (int b = 1; b < 5; ++b) {
                const uint32_t w = reinterpret_cast<const uint32_t *>(T[b - 1])[lane];
                uint32_t v = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) v |= (uint32_t)T[b - 1][(w >> (8 * j)) & 0xff] << (8 * j);
                __syncwarp();
                reinterpret_cast<uint32_t *>(T[b])[lane] = v;
                __syncwarp();
            }
            // ---- lane k takes the k-th sequence of the chain
            int pos = 0;
#pragma unroll
            for (int b = 0; b < 5; ++b)
                if ((lane >> b) & 1) pos = T[b][pos];
            const bool member = pos < kWin;
            const int nm = __popc(__ballot_sync(0xffffffffu, member));
            int4 q = make_int4(0, 0, 0, 0);
            int nx = 0;
            if (member) {
                q = cand[pos];
                nx = nextp[pos];
            }
            const int flags = q.w & ~0xffff;
            const bool term_in = flags & kTermIn, slow = flags & kSlow;
            const int off = member && !term_in && !slow
                                ? (int)__ldg(src + q.x + q.y) | ((int)__ldg(src + q.x + q.y + 1) << 8)
                                : 0;
            int len = member && !slow ? q.y + (term_in ? 0 : q.z) : 0;
            int incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int opl = op + incl - len, ms = opl + q.y;
            // ---- acceptance tests in sequence order (lz4.c:851-858, :868, :888-890)
            int stop = 0, epos = 0;  // 1: end of input, 2: malformed, 3: decode serially
            if (member) {
                if (slow) {
                    stop = 3;
                } else if (term_in || q.y > oend - opl - kMfLimit) {
                    if (q.y > oend - opl || q.y != iend - q.x) {
                        stop = 2;
                        epos = q.x;
                    } else {
                        stop = 1;
                    }
                } else if (off == 0 || off > ms) {
                    stop = 2;
                    epos = q.x + q.y + 2;
                } else if (q.z > oend - ms - kLastLiterals) {
                    stop = 2;
                    epos = nx;
                }
            }
            const unsigned sb = __ballot_sync(0xffffffffu, stop != 0);
            int ks = sb ? __ffs(sb) - 1 : nm;  // first sequence not taken as a plain one
            int kstop = __shfl_sync(0xffffffffu, stop, ks & 31);
            const int kepos = __shfl_sync(0xffffffffu, epos, ks & 31);
            // the window's output is staged in shared memory: sequences that
            // do not fit go to the serial path
            const unsigned fb = __ballot_sync(0xffffffffu, member && incl > kStage);
            if (fb && __ffs(fb) - 1 <= ks) {
                ks = __ffs(fb) - 1;
                kstop = 3;
            }
            // sequences [0, ks) are complete; sequence ks contributes its
            // literals when it ends the input
            const bool lits = lane < ks || (lane == ks && kstop == 1);
            const bool mat = lane < ks;
            if (lits && q.y <= 8) copy_lit(ring, opl, src + q.x, q.y);
            unsigned pend = __ballot_sync(0xffffffffu, lits && q.y > 8);
            while (pend) {
                const int who = __ffs(pend) - 1;
                pend &= pend - 1;
                const int o0 = __shfl_sync(0xffffffffu, opl, who);
                const int x0 = __shfl_sync(0xffffffffu, q.x, who);
                const int n0 = __shfl_sync(0xffffffffu, q.y, who);
                for (int k = lane; k < n0; k += 32) ring[(o0 + k) & kMask] = __ldg(src + x0 + k);
            }
            // matches whose sources lie before the window and are still in
            // the ring are copied by their lane; then, in rounds, every
            // short match whose source ends before the output of the first
            // match still to do (so that all of it is written) is copied by
            // its lane, and when there is none, that first match replays
            // with the whole warp (long matches, sources in global memory)
            const int lo = max(ring_lo, op + kStage - kRing);  // not overwritten by this window
            const bool fast_ring = mat && q.z <= 8 && ms - off + min(q.z, off) <= op && ms - off >= lo;
            const bool fast_old = mat && q.z <= 8 && ms - off + min(q.z, off) <= lo;
            const bool fast = fast_ring || fast_old;
            if (fast_ring) copy_match(ring, ms, off, q.z);
            else if (fast_old) copy_match_old(ring, ms, off, q.z, src, dst, hl);
            __syncwarp();
            bool todo = mat && !fast;
            pend = __ballot_sync(0xffffffffu, todo);
            while (pend) {
                const int who = __ffs(pend) - 1;
                const int m0 = __shfl_sync(0xffffffffu, ms, who);
                const bool ready = todo && q.z <= 8 && ms - off + min(q.z, off) <= m0 && ms - off >= lo;
                const unsigned rb = __ballot_sync(0xffffffffu, ready);
                if (rb) {  // includes `who` when it is short with its source in the ring
                    if (ready) {
                        copy_match(ring, ms, off, q.z);
                        todo = false;
                    }
                    pend &= ~rb;
                } else {
                    pend &= pend - 1;
                    if (lane == who) todo = false;
                    const int o0 = __shfl_sync(0xffffffffu, off, who);
                    const int l0 = __shfl_sync(0xffffffffu, q.z, who);
                    for (int k = lane; k < l0; k += 32) {
                        const int x = m0 - o0 + msrc(k, o0, l0);
                        ring[(m0 + k) & kMask] = out_byte(ring, src, dst, hl, x, lo);
                    }
                }
                __syncwarp();
            }
            const int nout = kstop == 1 ? __shfl_sync(0xffffffffu, opl + q.y, ks & 31) - op
                                        : (ks > 0 ? __shfl_sync(0xffffffffu, incl, ks - 1) : 0);
            {
                const int r = op & kMask, n1 = min(nout, kRing - r);
                flush(dst + op, ring, r, n1, lane);
                if (nout > n1) flush(dst + op + n1, ring, 0, nout - n1, lane);
            }
            __syncwarp();
            // ---- advance
            op += nout;
            if (kstop == 1) {
                done = true;
            } else if (kstop == 2) {
                err = kepos;
            } else if (kstop == 3) {
                // a sequence with long length fields, decoded serially
                int ip = __shfl_sync(0xffffffffu, s0 + pos, ks & 31);
                const int token = src[ip++];
                long long ll = token >> 4;
                if (ll == 15) ll += get_len(src, ip, iend);
                if (ll > (long long)(oend - op - kMfLimit) || ll > (long long)(iend - ip - (2 + 1 + kLastLiterals))) {
                    if (ll > (long long)(oend - op) || ll != (long long)(iend - ip)) {
                        err = ip;
                    } else {
                        lit_run(op, ip, (int)ll);
                        op += (int)ll;
                        done = true;
                    }
                } else {
                    lit_run(op, ip, (int)ll);
                    op += (int)ll;
                    ip += (int)ll;
                    const int o = (int)src[ip] | ((int)src[ip + 1] << 8);
                    ip += 2;
                    if (o == 0 || o > op) {
                        err = ip;
                    } else {
                        long long m = token & 15;
                        if (m == 15) m += get_len(src, ip, iend - (kLastLiterals + 1));
                        m += kMinMatch;
                        if (m > (long long)(oend - op - kLastLiterals)) {
                            err = ip;
                        } else {
                            __syncwarp();
                            for (int k = lane; k < (int)m; k += 32)
                                dst[op + k] = old_byte(src, dst, hl, op - o + msrc(k, o, (int)m));
                            __syncwarp();
                            op += (int)m;
                            s0 = ip;
                            ring_lo = op;  // written around the ring
                        }
                    }
                }
            } else {
                s0 = __shfl_sync(0xffffffffu, nx, nm - 1);
            }
            __syncwarp();
        }
        if (lane == 0) out_len[c] = err ? -err : op;
        __syncwarp();
    }
}

// n bytes from s to d by the CTA: bytes until d is 16-byte aligned, then
// 16-byte stores (each built from five 4-byte loads with funnel shifts), then
// the tail. Wide stores matter when the destination is host memory written
// over the CPU-GPU link. Reads up to 4 bytes past s + n.
__device__ __forceinline__ void cta_copy(uint8_t *__restrict__ d, const uint8_t *__restrict__ s, int n)
{
    if (n <= 0) return;
    int h = (int)((16 - (reinterpret_cast<uintptr_t>(d) & 15)) & 15);
    if (h > n) h = n;
    if ((int)threadIdx.x < h) d[threadIdx.x] = s[threadIdx.x];
    const uint8_t *s2 = s + h;
    uint4 *dw = reinterpret_cast<uint4 *>(d + h);
    const int m = n - h, nwd = m >> 4;
    const uint32_t sa = (uint32_t)(reinterpret_cast<uintptr_t>(s2) & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(s2 - sa);
    for (int i = threadIdx.x; i < nwd; i += blockDim.x) {
        const uint32_t *q = sw + 4 * i;
        const uint32_t a0 = q[0], a1 = q[1], a2 = q[2], a3 = q[3], a4 = sa ? q[4] : 0u;
        uint4 v;
        if (sa) {
            v.x = __funnelshift_r(a0, a1, 8 * sa);
            v.y = __funnelshift_r(a1, a2, 8 * sa);
            v.z = __funnelshift_r(a2, a3, 8 * sa);
            v.w = __funnelshift_r(a3, a4, 8 * sa);
        } else {
            v = make_uint4(a0, a1, a2, a3);
        }
        dw[i] = v;
    }
    const int t = m & 15;
    if ((int)threadIdx.x < t) d[h + 16 * nwd + threadIdx.x] = s2[16 * nwd + threadIdx.x];
}

// One CTA per chunk: the chunk's bytes to dst + dst_off[c]. With `hole`
// (LZ4 of block records), bytes [hole.x, hole.x + hole.z) of the chunk's
// output are the input bytes at hsrc + hsrc_off[c] + hole.y, which the
// encoder left unwritten.
__global__ void gather_kernel(const uint8_t *__restrict__ src, const long long *src_off, const int *len,
                              uint8_t *__restrict__ dst, const long long *dst_off, const int4 *hole,
                              const uint8_t *__restrict__ hsrc, const long long *hsrc_off)
{
    const int c = blockIdx.x;
    const int n = len[c];
    if (n <= 0) return;
    const uint8_t *s = src + src_off[c];
    uint8_t *d = dst + dst_off[c];
    const int4 hl = hole ? hole[c] : make_int4(0, 0, 0, 0);
    if (hl.z > 0) {
        cta_copy(d, s, hl.x);
        cta_copy(d + hl.x, hsrc + hsrc_off[c] + hl.y, hl.z);
        cta_copy(d + hl.x + hl.z, s + hl.x + hl.z, n - hl.x - hl.z);
    } else {
        cta_copy(d, s, n);
    }
}

}  // namespace cz

using namespace cz;

// kLzWarps chunks per CTA; 16 (512 threads, ~123 KB of shared memory)
// takes an SM, so that CTAs of this kernel and the wavelet kernel, which
// also takes a whole SM, share the machine SM by SM.
template <int W, bool SEQ, int E, int SW>
static cudaError_t launch_enc_t(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                uint8_t *out, const long long *out_off, int *out_len, int records, int grid,
                                cudaStream_t st, int4 *hole)
{
    const int sm = W <= 8 ? 0 : (int)sizeof(LzEncWarp<SW>) * W;
    auto k = lz4_encode_kernel<W, SEQ, E, SW>;
    if (sm > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e != cudaSuccess) return e;
    }
    k<<<grid, W * 32, sm, st>>>(in, in_off, in_len, nchunks, out, out_off, out_len, records, hole);
    return cudaGetLastError();
}

// one kernel per effort level, so that a level pays only for its own work
template <int W, bool SEQ, int SW>
static cudaError_t launch_enc_e(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                uint8_t *out, const long long *out_off, int *out_len, int records, int grid,
                                cudaStream_t st, int4 *hole, int effort)
{
    switch (effort) {
    case 0:
        return launch_enc_t<W, SEQ, 0, SW>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st,
                                           hole);
    case 2:
        return launch_enc_t<W, SEQ, 2, SW>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st,
                                           hole);
    default:
        return launch_enc_t<W, SEQ, 1, SW>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st,
                                           hole);
    }
}

// The super-window size depends only on the chunk count and the GPU, so
// that every CTA width writes the same bytes: 768 positions when all chunks
// fit on the SMs at once with 4 chunks per CTA (7 CTAs of 4 warps per SM),
// else 512.
static int window_for(int nchunks)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess)
        sms = 1;
    return (long long)nchunks <= 28LL * sms ? kWinLarge : kWinSmall;
}

template <int W, bool SEQ>
static cudaError_t launch_enc(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                              uint8_t *out, const long long *out_off, int *out_len, int records, int grid,
                              cudaStream_t st, int4 *hole, int effort)
{
    if (window_for(nchunks) == kWinLarge)
        return launch_enc_e<W, SEQ, kWinLarge>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st,
                                               hole, effort);
    return launch_enc_e<W, SEQ, kWinSmall>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st,
                                           hole, effort);
}

cudaError_t cz_launch_lz4_encode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, int *out_len, int records, int warps,
                                 int grid, cudaStream_t st, int4 *hole, int effort)
{
    if (nchunks <= 0) return cudaSuccess;
    switch (warps) {
    case 2:
        return launch_enc<2, false>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st, hole, effort);
    case 8:
        return launch_enc<8, false>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st, hole, effort);
    case 16:
        return launch_enc<16, false>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st, hole, effort);
    default:
        return launch_enc<4, false>(in, in_off, in_len, nchunks, out, out_off, out_len, records, grid, st, hole, effort);
    }
}

cudaError_t cz_launch_lz77_parse(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *seq, const long long *seq_off, int *seq_bytes, int records, int grid,
                                 cudaStream_t st, int effort)
{
    if (nchunks <= 0) return cudaSuccess;
    return launch_enc<4, true>(in, in_off, in_len, nchunks, seq, seq_off, seq_bytes, records, grid, st, nullptr, effort);
}

cudaError_t cz_launch_lz4_decode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, const int *out_cap, int *out_len, int grid,
                                 cudaStream_t st, int4 *hole)
{
    if (nchunks <= 0) return cudaSuccess;
    lz4_decode_kernel<<<grid, 128, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_cap, out_len, hole);
    return cudaGetLastError();
}

cudaError_t cz_launch_gather(const uint8_t *src, const long long *src_off, const int *len, int nchunks,
                             uint8_t *dst, const long long *dst_off, cudaStream_t st, const int4 *hole,
                             const uint8_t *hsrc, const long long *hsrc_off)
{
    if (nchunks <= 0) return cudaSuccess;
    gather_kernel<<<nchunks, 256, 0, st>>>(src, src_off, len, dst, dst_off, hole, hsrc, hsrc_off);
    return cudaGetLastError();
}
