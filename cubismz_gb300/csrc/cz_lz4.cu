// cz_lz4.cu -- LZ4 legacy block format on the GPU, one warp per chunk.
//
// Encoder: greedy parse, format-compatible with the reference decoder
// LZ4_uncompress_unknownOutputSize (ThirdParty/lz4/lz4.c:802-905): minimum
// match 4, offsets 1..65535, the last 5 bytes are literals and the last
// match starts at least 12 bytes before the end (lz4.c:177-204).
//   * Probe: a warp takes a 128-position window per step. Every lane loads
//     one aligned word (coalesced), takes the next word from its neighbour
//     and forms the 4-byte sequences of its 4 positions. The hash table
//     (2 Ki entries per warp, shared memory) stores position and sequence,
//     so candidates are verified without memory reads; repeats inside the
//     window are paired with __match_any_sync. Each lane then measures the
//     match length of its own candidates (up to 32 bytes; longer ones are
//     finished cooperatively when chosen).
//   * Select: the greedy walk through the window -- lowest position at or
//     after the cursor that has a match, take it, jump past it -- costs one
//     ballot per sequence; the window is never probed twice.
//   * Emit: sequences collect in a shared-memory batch; a flush sizes them
//     with a warp scan and lets every lane write one sequence (token,
//     lengths, short literals, offset); long literal runs are copied by the
//     whole warp.
//   * Windows without a match advance faster after 8 misses (the reference's
//     acceleration idea, lz4.c:389-393). Chunks made of block records
//     ([int32 nbytes][mask][4 byte planes], shuffle on) skip the search over
//     byte planes 1 and 2 -- the two middle mantissa bytes, which do not
//     compress -- and copy them as literals.
// Decoder: the same acceptance tests and error convention as
// LZ4_uncompress_unknownOutputSize (-(input position) on malformed input; an
// empty input yields 0). A walk over the tokens records a batch of
// sequences; literals of the batch are then copied in parallel and matches
// replayed in order, each by the whole warp (overlapping matches repeat
// their first `offset` bytes, the byte-serial copy semantics).
#include "cz_codec.h"

namespace cz {

constexpr int kLzWarps = 4;
constexpr int kHashLog = 10;
constexpr int kBatch = 256;  // sequences per decode batch
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
    if (sa == 0) {
        for (int i = lane; i < nw; i += 32) dw[i] = sw[i];
    } else {
        for (int i = lane; i < nw; i += 32) dw[i] = __funnelshift_r(sw[i], sw[i + 1], 8 * sa);
    }
    const int t = n & 3;
    if (lane < t) dst[4 * nw + lane] = src[4 * nw + lane];
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
//             insert, verification against the stored 4-byte sequence,
//             match length up to 12 bytes from memory; the result per
//             position goes to info[]: 0, or offset | (length-4) << 16 |
//             bit 31 when the match is longer than measured;
//   walk   -- lane k walks positions [base+64k, base+64k+64) greedily
//             (take the match at the cursor, jump past it, else step 1);
//   merge  -- lane k keeps its sequences that start at or after the end of
//             the last kept match of lanes < k: the kept matches never
//             overlap, so the parse stays valid LZ4 without any lane
//             waiting for another;
//   emit   -- every lane sizes its kept sequences, a warp scan places them,
//             every lane writes its own; literal runs longer than 32 bytes
//             are queued and copied by the whole warp.
constexpr int kSW = 2048, kSub = kSW / 32, kMaxSeqLane = kSub / 4;

// exact match length from (p, cand), starting `known` bytes in (lane-local)
__device__ __forceinline__ int match_len(const uint8_t *src, int p, int cand, int known, int matchlimit)
{
    int len = known;
    while (p + len < matchlimit) {
        const uint32_t x = rd32u(src + p + len) ^ rd32u(src + cand + len);
        if (x) {
            len += (__ffs(x) - 1) >> 3;
            break;
        }
        len += 4;
    }
    return len < matchlimit - p ? len : matchlimit - p;
}

__global__ void __launch_bounds__(kLzWarps * 32)
lz4_encode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, int *out_len, int records)
{
    __shared__ uint2 table_all[kLzWarps][1 << kHashLog];
    __shared__ uint32_t info_all[kLzWarps][kSW];
    __shared__ uint2 seq_all[kLzWarps][32][kMaxSeqLane];  // (start, off | (len-4) << 16), len < 2^15 else see lens
    __shared__ int lens_all[kLzWarps][32][kMaxSeqLane];
    __shared__ int4 longq_all[kLzWarps][64];  // (dst offset, src offset, n, -)
    __shared__ int nlong_all[kLzWarps];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint2 *table = table_all[wib];
    uint32_t *info = info_all[wib];
    uint2 *myseq = seq_all[wib][lane];
    int *mylen = lens_all[wib][lane];
    int4 *longq = longq_all[wib];
    int &nlong = nlong_all[wib];
    const int gw = blockIdx.x * kLzWarps + wib, nw = gridDim.x * kLzWarps;

    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int L = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int cap = L + L / 255 + 16;
        for (int i = lane; i < (1 << kHashLog); i += 32) table[i] = make_uint2(kEmpty, 0u);
        __syncwarp();
        int pos = 0, anchor = 0, op = 0, miss = 0;
        bool overflow = false;
        Skip sk;
        sk.on = records != 0;
        sk.next = 0;
        sk.lo = sk.hi = L + 1;
        if (sk.on) next_skip(sk, src, L);
        const int mflimit = L - kMfLimit, matchlimit = L - kLastLiterals;
        while (L >= kMfLimit + 1 && pos <= mflimit && !overflow) {
            if (pos >= sk.lo) {  // literal-only planes: jump over them
                if (pos < sk.hi) pos = sk.hi;
                next_skip(sk, src, L);
                miss = 0;
                continue;
            }
            const int base = pos;
            int end = base + kSW;
            if (end > mflimit + 1) end = mflimit + 1;
            if (end > sk.lo) end = sk.lo;
            // ---- probe [base, end)
            bool any_match = false;
            for (int wb = base & ~3; wb < end; wb += 128) {
                const int wpos = wb + 4 * lane;
                const uint32_t w0 = wpos + 4 <= L ? *reinterpret_cast<const uint32_t *>(src + wpos) : 0u;
                uint32_t w1 = __shfl_down_sync(0xffffffffu, w0, 1);
                if (lane == 31) w1 = wpos + 8 <= L ? *reinterpret_cast<const uint32_t *>(src + wpos + 4) : 0u;
                uint32_t seq[4], h[4];
                bool valid[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = wpos + j;
                    valid[j] = p >= base && p < end;
                    seq[j] = j ? __funnelshift_r(w0, w1, 8 * j) : w0;
                    h[j] = lz_hash(seq[j]);
                }
                uint2 e[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) e[j] = table[h[j]];
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (valid[j]) table[h[j]] = make_uint2((uint32_t)(wpos + j), seq[j]);
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = wpos + j;
                    const int cand = (int)e[j].x;
                    uint32_t v = 0;
                    if (valid[j] && e[j].x != kEmpty && e[j].y == seq[j] && cand < p && p - cand <= 65535) {
                        // up to 8 more bytes from memory; longer matches are finished in the walk
                        const int lim = matchlimit - p;
                        int len = kMinMatch;
                        const uint32_t x1 = rd32u(src + p + 4) ^ rd32u(src + cand + 4);
                        if (x1) {
                            len += (__ffs(x1) - 1) >> 3;
                        } else {
                            len += 4;
                            const uint32_t x2 = rd32u(src + p + 8) ^ rd32u(src + cand + 8);
                            len += x2 ? ((__ffs(x2) - 1) >> 3) : 4;
                        }
                        const bool more = len == 12 && len < lim;
                        if (len > lim) len = lim;
                        v = (uint32_t)(p - cand) | ((uint32_t)(len - kMinMatch) << 16) | (more ? 0x80000000u : 0u);
                    }
                    if (valid[j]) info[p - base] = v;
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
            // ---- walk: lane-local greedy parse of [base + 64*lane, +64)
            int ns = 0, first_start = 0x7fffffff, last_start = -1, last_end = -1;
            {
                const int w0p = base + kSub * lane;
                int q = w0p;
                const int qe = min(w0p + kSub, end);
                while (q < qe) {
                    const uint32_t v = info[q - base];
                    if (v) {
                        int len = kMinMatch + (int)((v >> 16) & 0x7fff);
                        const int off = (int)(v & 0xffff);
                        if (v & 0x80000000u) len = match_len(src, q, q - off, len, matchlimit);
                        myseq[ns] = make_uint2((uint32_t)q, (uint32_t)off);
                        mylen[ns] = len;
                        ++ns;
                        if (first_start > q) first_start = q;
                        last_start = q;
                        last_end = q + len;
                        q += len;
                    } else {
                        ++q;
                    }
                }
            }
            // ---- merge: P_k = end of the last kept match of lanes < k
            int P = anchor, myP = anchor;
            for (int k = 0; k < 32; ++k) {
                const int ls = __shfl_sync(0xffffffffu, last_start, k);
                const int le = __shfl_sync(0xffffffffu, last_end, k);
                if (lane == k) myP = P;
                if (ls >= P) P = le;
            }
            // ---- emit: kept sequences are those starting at or after myP
            int lit_from = myP, bytes = 0, nkeep = 0;
            for (int i = 0; i < ns; ++i) {
                const int st = (int)myseq[i].x;
                if (st < lit_from) continue;
                const int l = st - lit_from, ml = mylen[i] - kMinMatch;
                bytes += 1 + (l >= 15 ? len_bytes(l - 15) : 0) + l + 2 + (ml >= 15 ? len_bytes(ml - 15) : 0);
                lit_from = st + mylen[i];
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
            {
                int at = op + incl - bytes;
                lit_from = myP;
                for (int i = 0; i < ns; ++i) {
                    const int st = (int)myseq[i].x;
                    if (st < lit_from) continue;
                    const int l = st - lit_from, ml = mylen[i] - kMinMatch, off = (int)myseq[i].y;
                    uint8_t *d = dst + at;
                    *d++ = (uint8_t)(((l >= 15 ? 15 : l) << 4) | (ml >= 15 ? 15 : ml));
                    if (l >= 15) {
                        put_len_serial(d, l - 15);
                        d += len_bytes(l - 15);
                    }
                    if (l <= 32) {
                        for (int b = 0; b < l; ++b) d[b] = src[lit_from + b];
                    } else {
                        const int slot = atomicAdd(&nlong, 1);
                        if (slot < 64) longq[slot] = make_int4((int)(d - dst), lit_from, l, 0);
                    }
                    d += l;
                    d[0] = (uint8_t)off;
                    d[1] = (uint8_t)(off >> 8);
                    if (ml >= 15) put_len_serial(d + 2, ml - 15);
                    at += 1 + (l >= 15 ? len_bytes(l - 15) : 0) + l + 2 + (ml >= 15 ? len_bytes(ml - 15) : 0);
                    lit_from = st + mylen[i];
                }
            }
            __syncwarp();
            const int nl = nlong;
            if (nl > 64) {  // cannot happen: at most one long run per lane and 32 lanes
                overflow = true;
                break;
            }
            for (int i = 0; i < nl; ++i) {
                const int4 t = longq[i];
                warp_copy(dst + t.x, src + t.y, t.z, lane);
            }
            __syncwarp();
            op += total;
            anchor = P;
            pos = end > P ? end : P;
        }
        if (!overflow) {
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
                warp_copy(dst + op, src + anchor, lit, lane);
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

// Where the byte at output position s of a batch comes from: a literal of
// the batch, or a byte before the batch. Matches are followed back through
// their (periodic) sources; each step lands before the match it left.
__device__ __forceinline__ int resolve(const int4 *batch, int n, int batch_end, int s)
{
    const int b0 = batch[0].z;
    while (s >= b0) {
        int lo = 0, hi = n - 1;  // last sequence whose output starts at or before s
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (batch[mid].z <= s) lo = mid;
            else hi = mid - 1;
        }
        const int4 q = batch[lo];
        const int ms = q.z + q.y;
        if (s < ms) break;  // a literal of this batch
        s = ms - q.w + (s - ms) % q.w;
    }
    (void)batch_end;
    return s;
}

__global__ void __launch_bounds__(128)
lz4_decode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, const int *out_cap, int *out_len)
{
    // per warp: a batch of sequences (literal source, literal length,
    // output position, offset); a match runs to the next output position
    __shared__ int4 batch_all[4][kBatch + 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int4 *batch = batch_all[wib];
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int iend = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int oend = out_cap[c];
        int ip = 0, op = 0, err = 0, done = 0;
        if (iend <= 0) {
            if (lane == 0) out_len[c] = 0;  // lz4.c:836: error exit at position 0
            continue;
        }
        while (!done && !err) {
            // ---- token walk (lane 0)
            int n = 0, last_src = 0, last_len = 0;
            if (lane == 0) {
                while (n < kBatch) {
                    const int token = src[ip++];
                    long long len = token >> 4;
                    if (len == 15) len += get_len(src, ip, iend);
                    // lz4.c:851-858: the last sequence holds only literals and ends the input
                    if (len > (long long)(oend - op - kMfLimit) || len > (long long)(iend - ip - (2 + 1 + kLastLiterals))) {
                        if (len > (long long)(oend - op) || len != (long long)(iend - ip)) {
                            err = 1;
                        } else {
                            last_src = ip;
                            last_len = (int)len;
                            done = 1;
                        }
                        break;
                    }
                    const int lsrc = ip, lpos = op;
                    op += (int)len;
                    ip += (int)len;
                    const int off = (int)src[ip] | ((int)src[ip + 1] << 8);
                    ip += 2;
                    if (off == 0 || off > op) {
                        err = 1;
                        break;
                    }
                    long long ml = token & 15;
                    if (ml == 15) ml += get_len(src, ip, iend - (kLastLiterals + 1));  // lz4.c:873-882
                    ml += kMinMatch;
                    if (ml > (long long)(oend - op - kLastLiterals)) {  // lz4.c:888-890
                        err = 1;
                        break;
                    }
                    batch[n++] = make_int4(lsrc, (int)len, lpos, off);
                    op += (int)ml;
                }
                batch[n] = make_int4(0, 0, op, 1);  // sentinel: end of the last match
            }
            n = __shfl_sync(0xffffffffu, n, 0);
            ip = __shfl_sync(0xffffffffu, ip, 0);
            op = __shfl_sync(0xffffffffu, op, 0);
            err = __shfl_sync(0xffffffffu, err, 0);
            done = __shfl_sync(0xffffffffu, done, 0);
            last_src = __shfl_sync(0xffffffffu, last_src, 0);
            last_len = __shfl_sync(0xffffffffu, last_len, 0);
            __syncwarp();
            if (err) break;
            // ---- literals: one sequence per lane, long runs by the warp
            for (int b0 = 0; b0 < n; b0 += 32) {
                const int k = b0 + lane;
                int4 q = make_int4(0, 0, 0, 1);
                if (k < n) q = batch[k];
                if (q.y <= 32) {
                    for (int i = 0; i < q.y; ++i) dst[q.z + i] = src[q.x + i];
                }
                unsigned pend = __ballot_sync(0xffffffffu, q.y > 32);
                while (pend) {
                    const int who = __ffs(pend) - 1;
                    pend &= pend - 1;
                    const int xs = __shfl_sync(0xffffffffu, q.x, who);
                    const int yl = __shfl_sync(0xffffffffu, q.y, who);
                    const int zp = __shfl_sync(0xffffffffu, q.z, who);
                    warp_copy(dst + zp, src + xs, yl, lane);
                }
            }
            __syncwarp();
            // ---- matches: every byte resolves its source independently
            for (int b0 = 0; b0 < n; b0 += 32) {
                const int k = b0 + lane;
                int ms = 0, me = 0, off = 1;
                if (k < n) {
                    const int4 q = batch[k];
                    ms = q.z + q.y;
                    me = batch[k + 1].z;
                    off = q.w;
                }
                if (me - ms <= 32) {
                    for (int t = ms; t < me; ++t) dst[t] = __ldcg(dst + resolve(batch, n, op, t - off));
                }
                unsigned pend = __ballot_sync(0xffffffffu, me - ms > 32);
                while (pend) {
                    const int who = __ffs(pend) - 1;
                    pend &= pend - 1;
                    const int s0 = __shfl_sync(0xffffffffu, ms, who);
                    const int e0 = __shfl_sync(0xffffffffu, me, who);
                    const int o0 = __shfl_sync(0xffffffffu, off, who);
                    for (int t = s0 + lane; t < e0; t += 32) dst[t] = __ldcg(dst + resolve(batch, n, op, t - o0));
                }
            }
            __syncwarp();
            if (done) {
                for (int i = lane; i < last_len; i += 32) dst[op + i] = src[last_src + i];
                op += last_len;
            }
        }
        if (lane == 0) out_len[c] = err ? -(ip > 0 ? ip : 1) : op;
        __syncwarp();
    }
}

__global__ void gather_kernel(const uint8_t *__restrict__ src, const long long *src_off, const int *len,
                              uint8_t *__restrict__ dst, const long long *dst_off)
{
    const int c = blockIdx.x;
    const int n = len[c];
    const uint8_t *s = src + src_off[c];
    uint8_t *d = dst + dst_off[c];
    // 4-byte stores once d is aligned
    int h = (int)((4 - (reinterpret_cast<uintptr_t>(d) & 3)) & 3);
    if (h > n) h = n;
    if ((int)threadIdx.x < h) d[threadIdx.x] = s[threadIdx.x];
    const uint8_t *s2 = s + h;
    uint32_t *dw = reinterpret_cast<uint32_t *>(d + h);
    const int m = n - h, nwd = m >> 2;
    const uint32_t sa = (uint32_t)(reinterpret_cast<uintptr_t>(s2) & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(s2 - sa);
    for (int i = threadIdx.x; i < nwd; i += blockDim.x) dw[i] = sa ? __funnelshift_r(sw[i], sw[i + 1], 8 * sa) : sw[i];
    const int t = m & 3;
    if ((int)threadIdx.x < t) d[h + 4 * nwd + threadIdx.x] = s2[4 * nwd + threadIdx.x];
}

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_lz4_encode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, int *out_len, int records, int grid,
                                 cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    lz4_encode_kernel<<<grid, kLzWarps * 32, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_len, records);
    return cudaGetLastError();
}

cudaError_t cz_launch_lz4_decode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, const int *out_cap, int *out_len, int grid,
                                 cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    lz4_decode_kernel<<<grid, 128, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_cap, out_len);
    return cudaGetLastError();
}

cudaError_t cz_launch_gather(const uint8_t *src, const long long *src_off, const int *len, int nchunks,
                             uint8_t *dst, const long long *dst_off, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    gather_kernel<<<nchunks, 256, 0, st>>>(src, src_off, len, dst, dst_off);
    return cudaGetLastError();
}
