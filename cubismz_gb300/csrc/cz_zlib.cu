// cz_zlib.cu -- zlib streams (RFC 1950 wrapper, RFC 1951 DEFLATE), the
// format of the reference's zlib encoder (deflateInit/deflate with Z_FINISH,
// CompressionEncoders.h:116-190) and decoder (inflateInit/inflate,
// CompressionEncoders.h:48-88).
//
// Encoder (deflate_kernel): one warp per chunk, fed by the LZ77 parse of the
// LZ4 encoder run with a 32 KiB window (cz_lz4.cu, SEQ mode). A chunk of
// shuffled block records gets a DEFLATE block per record mask and byte
// plane (other chunks one per 64 KiB): per block, the warp counts the
// symbols of the items that start in it (literal bytes with one
// shared-memory add per distinct byte of 32; matches of more than 258 bytes
// in pieces), sorts the used symbols (bitonic, by frequency), one lane
// builds the length-limited codes (cz_deflate.cuh), and the exact sizes of
// the stored, fixed and dynamic codings pick the smallest; then 32 items per
// step (a literal or a match piece each), a warp scan of their bit counts,
// and OR-writes into a per-warp ring of words that is flushed to the output
// with word stores. zlib header 78 9C, Adler-32 by a warp reduction.
//
// Decoder (inflate_kernel): one warp per chunk. Lane 0 reads the header and
// the blocks (stored, fixed Huffman, dynamic Huffman) and decodes symbols
// with 10-bit lookup tables (longer codes by the canonical walk); literals
// go straight to the output, matches into a batch. The warp then writes all
// of the batch's match bytes in parallel, each following its source back
// through earlier matches of the batch to a byte written before. The Adler-32
// of the output is a warp reduction, checked against the trailer. Malformed
// input (bad header, code lengths, symbols, distances past the start, output
// past the capacity, truncated input or a wrong checksum) gives a negative
// length; every read and write is bounds checked.
#include "cz_codec.h"
#include "cz_deflate.cuh"

namespace cz {

using namespace zl;

constexpr int kZBatch = 128;  // matches per batch

// n bytes from s to d by the warp (4-byte stores once d is aligned); every
// load is of an aligned word holding at least one byte of the run.
__device__ __forceinline__ void run_copy(uint8_t *d, const uint8_t *s, int n, int lane)
{
    int h = (int)((4 - (reinterpret_cast<uintptr_t>(d) & 3)) & 3);
    if (h > n) h = n;
    if (lane < h) d[lane] = s[lane];
    d += h;
    s += h;
    n -= h;
    const int nw = n >> 2;
    const uint32_t sa = (uint32_t)(reinterpret_cast<uintptr_t>(s) & 3);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(s - sa);
    uint32_t *dw = reinterpret_cast<uint32_t *>(d);
    for (int i = lane; i < nw; i += 32) dw[i] = sa ? __funnelshift_r(sw[i], sw[i + 1], 8 * sa) : sw[i];
    const int t = n & 3;
    if (lane < t) d[4 * nw + lane] = s[4 * nw + lane];
}

__global__ void __launch_bounds__(32)
inflate_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
               uint8_t *__restrict__ out, const long long *out_off, const int *out_cap, int *out_len)
{
    __shared__ Huff lit, dist;
    __shared__ unsigned char lens[320];
    __shared__ int batch[kZBatch][3];  // matches: output position, length, distance
    __shared__ int mpre[kZBatch + 1];  // exclusive prefix of the match lengths
    __shared__ int s_state[4];         // matches in the batch, error, done, Adler-32 of the trailer
    __shared__ long long s_run[3];     // a stored block: input position, output position, length
    const int lane = threadIdx.x;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint8_t *src = in + in_off[c];
        uint8_t *dst = out + out_off[c];
        const long long oend = out_cap[c];
        Inflater z;  // lane 0's decoder state, kept in registers across batches
        if (lane == 0) z.start(src, in_len[c]);
        for (;;) {
            if (lane == 0) {
                s_state[0] = z.step(dst, oend, batch, kZBatch, lit, dist, lens);
                s_state[1] = z.err;
                s_state[2] = z.done();
                s_run[0] = z.run_src;
                s_run[1] = z.run_dst;
                s_run[2] = z.err ? 0 : z.run_n;
            }
            __syncwarp();
            if (s_run[2] > 0) run_copy(dst + s_run[1], src + s_run[0], (int)s_run[2], lane);
            // the batch's match bytes, all in parallel: byte k of a match at p
            // with distance d is out[p - d + (k mod d)]; where that lies in an
            // earlier match of the batch (or this one) the source is followed
            // back until it is a byte written before the replay (a literal of
            // the batch or earlier output)
            const int n = s_state[0];
            {
                int incl = 0;
                for (int i0 = 0; i0 < n; i0 += 32) {  // exclusive prefix of the match lengths (warp-uniform loop)
                    const int i = i0 + lane;
                    const int v = i < n ? batch[i][1] : 0;
                    int x = v;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int t = __shfl_up_sync(0xffffffffu, x, o);
                        if (lane >= o) x += t;
                    }
                    if (i < n) mpre[i] = incl + x - v;
                    incl += __shfl_sync(0xffffffffu, x, 31);
                }
                if (lane == 0) mpre[n] = incl;
            }
            __syncwarp();
            const int mtotal = mpre[n];
            for (int t = lane; t < mtotal; t += 32) {
                int i = 0;  // match holding byte t of the batch's match bytes
#pragma unroll
                for (int step = 64; step; step >>= 1)
                    if (i + step < n && mpre[i + step] <= t) i += step;
                const int y = batch[i][0] + t - mpre[i];
                int x = y;
                for (int hop = 0; hop <= n; ++hop) {
                    int j = 0;  // last match starting at or before x
#pragma unroll
                    for (int step = 64; step; step >>= 1)
                        if (j + step < n && batch[j + step][0] <= x) j += step;
                    const int pj = batch[j][0], lj = batch[j][1], dj = batch[j][2];
                    if (x < pj || x >= pj + lj) break;
                    x = pj - dj + (dj >= lj ? x - pj : (x - pj) % dj);
                }
                dst[y] = __ldcg(dst + x);
            }
            __syncwarp();
            const int e = s_state[1], dn = s_state[2];
            __syncwarp();
            if (e || dn) break;
        }
        // Adler-32 of the output (A = 1 + sum d_i, B = n + sum (n - i) d_i,
        // mod 65521) against the trailer
        if (lane == 0) {
            if (!z.err) s_state[3] = (int)z.trailer();
            s_state[1] = z.err;
            s_state[0] = (int)z.op;
        }
        __syncwarp();
        int e = s_state[1];
        const long long total = s_state[0];
        if (!e) {
            unsigned long long sa = 0, sb = 0;
            for (long long i = lane; i < total; i += 32) {
                const unsigned v = __ldcg(dst + i);
                sa += v;
                sb += (unsigned long long)(total - i) * v;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sa += __shfl_xor_sync(0xffffffffu, sa, o);
                sb += __shfl_xor_sync(0xffffffffu, sb, o);
            }
            const unsigned A = (unsigned)((1 + sa) % 65521ull);
            const unsigned B = (unsigned)(((unsigned long long)total + sb) % 65521ull);
            if (((B << 16) | A) != (unsigned)s_state[3]) e = 22;
        }
        if (lane == 0) out_len[c] = e ? -e : (int)total;
        __syncwarp();
    }
}

// ---------------------------------------------------------------- encoder
constexpr int kZWarps = 4;     // chunks per CTA
constexpr int kRingW = 512;    // bit-ring words per warp
constexpr int kRingM = kRingW - 1;

struct DeflateWarp {
    uint32_t lf[288], df[32];
    Codes codes;
    union {
        uint32_t ring[kRingW];
        struct {  // code construction
            uint32_t key[512];  // (weight << 9 | symbol), sorted; unused: ~0
            uint32_t w[288], iw[288];
            uint16_t sym[288], par[576], dep[576];
            uint8_t l[288];
        } b;
    } u;
    int beg[32], end[32], litpos[32], nlit[32], mstart[32], mlen[32], dist[32], k0[32];
    int state[4];
};

// Code lengths for freq[0..n) into len: the warp sorts the used symbols by
// (frequency, symbol) -- a bitonic sort of keys weight << 9 | symbol over 512
// slots (block counts stay below 2^22) -- and lane 0 runs huff_lengths.
// False if it fails.
__device__ bool warp_code(DeflateWarp &s, const uint32_t *freq, int n, uint8_t *len, int lane)
{
    auto &b = s.u.b;
    int used = 0;
    for (int x = lane; x < n; x += 32) used += freq[x] != 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) used += __shfl_xor_sync(0xffffffffu, used, o);
    // at least two codes: the lowest unused symbols get weight one (never sent)
    int need = used < 2 ? 2 - used : 0;
    for (int x0 = 0; x0 < 512; x0 += 32) {
        const int x = x0 + lane;
        uint32_t f = x < n ? freq[x] : 0u;
        const bool zero = x < n && f == 0u;
        const unsigned zb = __ballot_sync(0xffffffffu, zero);
        if (zero && need > 0 && __popc(zb & ((1u << lane) - 1u)) < need) f = 1u;
        need -= min(need, __popc(zb));
        b.key[x] = f ? (f << 9 | (uint32_t)x) : 0xffffffffu;
    }
    used = max(used, 2);
    __syncwarp();
    // bitonic sort, ascending, 256 compare-exchanges per pass
    for (int k = 2; k <= 512; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < 256; i += 32) {
                const int lo = ((i & ~(j - 1)) << 1) | (i & (j - 1)), hi = lo + j;
                const uint32_t a = b.key[lo], c = b.key[hi];
                const bool up = (lo & k) == 0;
                if ((a > c) == up) {
                    b.key[lo] = c;
                    b.key[hi] = a;
                }
            }
            __syncwarp();
        }
    }
    for (int x = lane; x < n; x += 32) len[x] = 0;
    for (int r = lane; r < used; r += 32) {
        const uint32_t kk = b.key[r];
        b.sym[r] = (uint16_t)(kk & 511u);
        b.w[r] = kk >> 9;
    }
    __syncwarp();
    int ok = 1;
    if (lane == 0) {
        ok = zl::huff_lengths(b.w, used, zl::kMaxLit, b.l, b.iw, b.par, b.dep) ? 1 : 0;
        if (ok)
            for (int i = 0; i < used; ++i) len[b.sym[i]] = b.l[i];
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
}

// zl::data_bits (with the dynamic lengths) and zl::fixed_block_bits of the
// block's counts, summed by the warp instead of lane 0; the same integers.
__device__ void warp_block_bits(const DeflateWarp &s, const uint8_t *llen, const uint8_t *dlen, int lane,
                                long long &data, long long &fixed)
{
    long long a = 0, f = 0;
    for (int x = lane; x < zl::kLitSyms; x += 32) {
        const long long c = s.lf[x];
        a += c * llen[x];
        f += c * zl::fixed_lit_len(x);
    }
    if (lane < 29) {
        const long long c = s.lf[257 + lane];
        a += c * zl::len_extra(lane);
        f += c * zl::len_extra(lane);
    }
    if (lane < zl::kDistSyms) {
        const long long c = s.df[lane];
        a += c * (dlen[lane] + zl::dist_extra(lane));
        f += c * (5 + zl::dist_extra(lane));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        f += __shfl_xor_sync(0xffffffffu, f, o);
    }
    data = a;
    fixed = 3 + f;
}

// Serial bit writer of lane 0 into the ring (block headers).
struct RingW {
    uint32_t *ring;
    int bp;
    __device__ void put(unsigned long long v, int n)
    {
        const int sh = bp & 31, wi = bp >> 5;
        const unsigned long long lo = v << sh;
        ring[wi & kRingM] |= (uint32_t)lo;
        ring[(wi + 1) & kRingM] |= (uint32_t)(lo >> 32);
        if (sh && n + sh > 64) ring[(wi + 2) & kRingM] |= (uint32_t)(v >> (64 - sh));
        bp += n;
    }
};

__device__ __forceinline__ void ring_or(uint32_t *ring, int b, unsigned long long v)
{
    const int sh = b & 31, wi = b >> 5;
    const unsigned long long lo = v << sh;
    const uint32_t x0 = (uint32_t)lo, x1 = (uint32_t)(lo >> 32), x2 = sh ? (uint32_t)(v >> (64 - sh)) : 0u;
    if (x0) atomicOr(ring + (wi & kRingM), x0);
    if (x1) atomicOr(ring + ((wi + 1) & kRingM), x1);
    if (x2) atomicOr(ring + ((wi + 2) & kRingM), x2);
}

// The ring of one chunk's output: words [flushed, bp/32] are live; older
// words are in the output, their slots zero. Flushes keep a step of at most
// 32 items (48 bits each) clear of the live words.
struct Ring {
    uint32_t *ring, *dstw;
    int bp, flushed, wlimit;
    __device__ void flush_to(int to, int lane)
    {
        for (int w = flushed + lane; w < to; w += 32) {
            if (w < wlimit) dstw[w] = ring[w & kRingM];
            ring[w & kRingM] = 0;
        }
        flushed = to;
        __syncwarp();
    }
    __device__ void make_room(int lane, int words = 52)
    {
        if ((bp >> 5) + words >= flushed + kRingW) flush_to(bp >> 5, lane);
    }
};

// Index j of the batch entry whose [beg, end) holds item t (t < end[31]).
__device__ __forceinline__ int find_item(const int *end, int t)
{
    int j = 0;
#pragma unroll
    for (int step = 16; step; step >>= 1)
        if (end[j + step - 1] <= t) j += step;
    return j;
}

// Sequence cursor: record index and the input position of its literals.
struct Cursor {
    int i, pos;
};

// The items (literal bytes and match pieces) of the parse that start in
// [lo, hi), from cursor cur, 32 sequences per batch and 32 items per step.
// MODE 0 counts symbols into s.lf/s.df and returns the end of the bytes the
// items cover; MODE 1 writes their codes into the ring. `next` is set to
// the first sequence that reaches past that end.
template <int MODE>
__device__ int block_items(DeflateWarp &s, const unsigned long long *seq, int nseq, Cursor cur, int lo, int hi,
                           const uint8_t *src, Ring *rg, Cursor *next, int lane)
{
    int cov = lo;
    int i0 = cur.i, pos = cur.pos;
    for (;;) {
        const int i = i0 + lane;
        const unsigned long long r = i < nseq ? seq[i] : 0ull;
        const int lit = zl::seq_lit(r), m = zl::seq_mlen(r), d = zl::seq_dist(r);
        const int span = lit + m;
        int incl = span;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int ls = pos + incl - span, ms = ls + lit;
        const int span_total = __shfl_sync(0xffffffffu, incl, 31);
        // literal sub-range [a, b) and pieces [k0, k1) that start in [lo, hi)
        const int a = min(max(lo - ls, 0), lit), b = min(max(hi - ls, 0), lit);
        const int k0 = m ? zl::pieces_before(m, lo - ms) : 0, k1 = m ? zl::pieces_before(m, hi - ms) : 0;
        const int nl = b - a, np = k1 - k0, items = nl + np;
        int c = 0;
        if (np > 0) c = ms + zl::piece_start(m, k1 - 1) + zl::piece_len(m, k1 - 1);
        else if (nl > 0) c = ls + b;
#pragma unroll
        for (int o = 16; o; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
        cov = max(cov, c);
        int ii = items;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, ii, o);
            if (lane >= o) ii += t;
        }
        s.end[lane] = ii;
        s.beg[lane] = ii - items;
        s.litpos[lane] = ls + a;
        s.nlit[lane] = nl;
        s.mstart[lane] = ms;
        s.mlen[lane] = m;
        s.dist[lane] = d;
        s.k0[lane] = k0;
        const int total = __shfl_sync(0xffffffffu, ii, 31);
        __syncwarp();
        // kU steps of 32 items at a time: their literal bytes are loaded
        // together, then the steps are counted or written in order
        constexpr int kU = 4;
        for (int t0 = 0; t0 < total; t0 += 32 * kU) {
            if (MODE == 1) rg->make_room(lane, 48 * kU + 4);
            int byte[kU], nb[kU];  // byte >= 256: not a literal (inactive lanes never group)
            unsigned long long v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = t0 + 32 * u + lane;
                byte[u] = 256 + lane;
                nb[u] = 0;
                v[u] = 0;
                if (t < total) {
                    const int j = find_item(s.end, t);
                    const int k = t - s.beg[j];
                    if (k < s.nlit[j]) {
                        byte[u] = src[s.litpos[j] + k];
                    } else {
                        const int mj = s.mlen[j], pk = s.k0[j] + k - s.nlit[j];
                        const int pl = zl::piece_len(mj, pk);
                        if (MODE == 0) {
                            atomicAdd(&s.lf[257 + zl::len_sym(pl)], 1u);
                            atomicAdd(&s.df[zl::dist_sym(s.dist[j])], 1u);
                        } else {
                            nb[u] = zl::match_bits(s.codes, pl, s.dist[j], v[u]);
                        }
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                if (MODE == 0) {
                    const unsigned grp = __match_any_sync(0xffffffffu, byte[u]);
                    if (byte[u] < 256 && lane == __ffs(grp) - 1) atomicAdd(&s.lf[byte[u]], (unsigned)__popc(grp));
                } else {
                    if (byte[u] < 256) {
                        v[u] = s.codes.lcode[byte[u]];
                        nb[u] = s.codes.llen[byte[u]];
                    }
                    int bi = nb[u];
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int w = __shfl_up_sync(0xffffffffu, bi, o);
                        if (lane >= o) bi += w;
                    }
                    if (nb[u]) ring_or(rg->ring, rg->bp + bi - nb[u], v[u]);
                    rg->bp += __shfl_sync(0xffffffffu, bi, 31);
                }
            }
            if (MODE == 1) __syncwarp();  // the next flush reads these words
        }
        __syncwarp();
        const bool last = pos + span_total >= hi || i0 + 32 >= nseq;
        if (last) {
            // the next block starts at the first sequence reaching past cov
            const int cv = __shfl_sync(0xffffffffu, cov, 0);
            const unsigned beyond = __ballot_sync(0xffffffffu, i < nseq && ls + span > cv);
            if (beyond) {
                const int f = __ffs(beyond) - 1;
                next->i = i0 + f;
                next->pos = __shfl_sync(0xffffffffu, ls, f);
            } else {
                next->i = min(i0 + 32, nseq);
                next->pos = pos + span_total;
            }
            return cv;
        }
        pos += span_total;
        i0 += 32;
    }
}

// Validation of a chunk's parse: lengths sum to L, matches of at least 3
// bytes within the window and the output so far.
__device__ bool parse_ok(const unsigned long long *seq, int nseq, int L, int lane)
{
    int pos = 0;
    bool ok = true;
    for (int i0 = 0; i0 < nseq; i0 += 32) {
        const int i = i0 + lane;
        const unsigned long long r = i < nseq ? seq[i] : 0ull;
        const int lit = zl::seq_lit(r), m = zl::seq_mlen(r), d = zl::seq_dist(r);
        int incl = lit + m;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int ms = pos + incl - m;
        ok = ok && (m == 0 || (m >= 3 && d >= 1 && d <= zl::kMaxDist && d <= ms));
        pos += __shfl_sync(0xffffffffu, incl, 31);
        if (pos > L) ok = false;
    }
    return __all_sync(0xffffffffu, ok) && pos == L;
}

__global__ void __launch_bounds__(kZWarps * 32)
deflate_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len,
               const uint8_t *__restrict__ sq, const long long *seq_off, const int *seq_bytes, int nchunks,
               int records, uint8_t *__restrict__ out, long long out_slot, long long *out_off, int *out_len)
{
    __shared__ DeflateWarp sw[kZWarps];
    const int lane = threadIdx.x & 31;
    DeflateWarp &s = sw[threadIdx.x >> 5];
    const int gw = blockIdx.x * kZWarps + (threadIdx.x >> 5), nw = gridDim.x * kZWarps;
    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int L = in_len[c];
        const int sb = seq_bytes[c];
        const unsigned long long *seq = reinterpret_cast<const unsigned long long *>(sq + seq_off[c]);
        const int nseq = sb >= 8 && (sb & 7) == 0 ? sb / 8 : 0;
        uint8_t *dst = out + (long long)c * out_slot;
        if (lane == 0) out_off[c] = (long long)c * out_slot;
        if (nseq == 0 || !parse_ok(seq, nseq, L, lane)) {
            if (lane == 0) out_len[c] = -1;
            __syncwarp();
            continue;
        }
        // Adler-32 of the input
        unsigned long long sa = 0, sbs = 0;
        for (int i = lane; i < L; i += 32) {
            const unsigned v = src[i];
            sa += v;
            sbs += (unsigned long long)(L - i) * v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_xor_sync(0xffffffffu, sa, o);
            sbs += __shfl_xor_sync(0xffffffffu, sbs, o);
        }
        const unsigned adler =
            ((unsigned)(((unsigned long long)L + sbs) % 65521ull) << 16) | (unsigned)((1 + sa) % 65521ull);
        Ring rg{s.u.ring, reinterpret_cast<uint32_t *>(dst), 16, 0, (int)(out_slot / 4)};
        zl::Bounds bnd;
        bnd.init(src, L, records != 0);
        Cursor cur{0, 0};
        int lo = 0, err = 0, nblk = 0;
        bool first = true;
        for (;;) {
            const int hi = bnd.next(lo);
            // ---- pass 1: symbol counts of the items starting in [lo, hi)
            for (int x = lane; x < 288; x += 32) s.lf[x] = x == 256 ? 1u : 0u;
            s.df[lane] = 0;
            __syncwarp();
            Cursor nxt;
            const int cov = block_items<0>(s, seq, nseq, cur, lo, hi, src, nullptr, &nxt, lane);
            const bool final = cov >= L;
            // ---- codes; the block coding with the fewest bits
            // (the code construction borrows the ring: flush it first)
            if (!first) rg.flush_to(rg.bp >> 5, lane);
            const uint32_t keep = first ? 0x9c78u : s.u.ring[rg.flushed & kRingM];  // zlib header / partial word
            __syncwarp();  // read before the code construction overwrites the ring
            bool ok = warp_code(s, s.lf, zl::kLitSyms, s.codes.llen, lane);
            ok = warp_code(s, s.df, zl::kDistSyms, s.codes.dlen, lane) && ok;
            long long dbits, fbits;
            warp_block_bits(s, s.codes.llen, s.codes.dlen, lane, dbits, fbits);
            if (lane == 0) {
                Codes &cd = s.codes;
                for (int x = zl::kLitSyms; x < 288; ++x) cd.llen[x] = 0;
                for (int x = zl::kDistSyms; x < 32; ++x) cd.dlen[x] = 0;
                long long dyn = -1;
                if (ok) {
                    zl::canon_codes(cd.llen, 288, cd.lcode);
                    zl::canon_codes(cd.dlen, 32, cd.dcode);
                    const long long hb = zl::dynamic_header(cd);
                    if (hb >= 0) dyn = hb + dbits;
                }
                const long long fix = fbits;
                const long long sto = cov - lo <= zl::kStoredMax ? zl::stored_block_bits(rg.bp, cov - lo) : -1;
                int mode = 2;
                long long best = dyn;
                if (dyn < 0 || fix <= dyn) {
                    mode = 1;
                    best = fix;
                }
                if (sto >= 0 && sto <= best) {
                    mode = 0;
                    best = sto;
                }
                if (mode == 1) zl::fixed_codes(cd);
                s.state[0] = mode;
                s.state[2] = (int)best;
            }
            __syncwarp();
            for (int w = lane; w < kRingW; w += 32) s.u.ring[w] = 0;
            __syncwarp();
            if (lane == 0) s.u.ring[rg.flushed & kRingM] = keep;
            __syncwarp();
            const int mode = s.state[0], bp0 = rg.bp;
            // ---- pass 2: the block
            if (mode == 0) {
                if (lane == 0) {
                    RingW wr{s.u.ring, rg.bp};
                    wr.put(final ? 1u : 0u, 3);
                    wr.bp = (wr.bp + 7) & ~7;
                    const unsigned n = (unsigned)(cov - lo);
                    wr.put(n | (~n & 0xffffu) << 16, 32);
                    s.state[1] = wr.bp;
                }
                __syncwarp();
                rg.bp = s.state[1];
                for (int t0 = 0; t0 < cov - lo; t0 += 32) {
                    rg.make_room(lane);
                    const int t = t0 + lane;
                    if (t < cov - lo) ring_or(rg.ring, rg.bp + 8 * lane, src[lo + t]);
                    rg.bp += 8 * min(32, cov - lo - t0);
                    __syncwarp();
                }
            } else {
                if (lane == 0) {
                    RingW wr{s.u.ring, rg.bp};
                    if (mode == 1) wr.put((final ? 1u : 0u) | 1u << 1, 3);
                    else zl::put_dynamic_header(wr, s.codes, final);
                    s.state[1] = wr.bp;
                }
                __syncwarp();
                rg.bp = s.state[1];
                Cursor dummy;
                block_items<1>(s, seq, nseq, cur, lo, hi, src, &rg, &dummy, lane);
                rg.make_room(lane);
                if (lane == 0) ring_or(rg.ring, rg.bp, s.codes.lcode[256]);
                rg.bp += s.codes.llen[256];
                __syncwarp();
            }
            first = false;
            if (rg.bp - bp0 != s.state[2]) err = 2;  // written bits must be the counted ones
            if (!final && cov <= lo) err = 3;         // every block makes progress
            if (++nblk > L / zl::kMinBlock + 2) err = 4;
            cur = nxt;
            lo = cov;
            if (final || err) break;
        }
        rg.flush_to((rg.bp + 31) >> 5, lane);
        const int nbytes = (rg.bp + 7) >> 3;
        if (lane == 0) {
            if (err || nbytes + 4 > out_slot) {
                out_len[c] = -2;
            } else {
                dst[nbytes] = (uint8_t)(adler >> 24);
                dst[nbytes + 1] = (uint8_t)(adler >> 16);
                dst[nbytes + 2] = (uint8_t)(adler >> 8);
                dst[nbytes + 3] = (uint8_t)adler;
                out_len[c] = nbytes + 4;
            }
        }
        __syncwarp();
    }
}

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_deflate(const uint8_t *in, const long long *in_off, const int *in_len, const uint8_t *seq,
                              const long long *seq_off, const int *seq_bytes, int nchunks, int records, uint8_t *out,
                              long long out_slot, long long *out_off, int *out_len, int grid, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    deflate_kernel<<<grid, kZWarps * 32, 0, st>>>(in, in_off, in_len, seq, seq_off, seq_bytes, nchunks, records,
                                                  out, out_slot, out_off, out_len);
    return cudaGetLastError();
}

cudaError_t cz_launch_inflate(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks, uint8_t *out,
                              const long long *out_off, const int *out_cap, int *out_len, int grid, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    inflate_kernel<<<grid, 32, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_cap, out_len);
    return cudaGetLastError();
}
