// cz_inflate.cuh -- the serial part of zlib decoding (RFC 1950 wrapper, RFC
// 1951 DEFLATE), shared by the GPU kernel (run by one lane per chunk) and the
// host test harness: bit reader, canonical Huffman codes, and the decoder
// state machine that writes literals and records matches in batches.
//
// The length and distance tables of RFC 1951 3.2.5 are computed from their
// closed forms; the code-length code order of 3.2.7 is packed in constants.
#pragma once
#include <stdint.h>

#include "cz_arith.cuh"  // CZ_HD

// member functions (CZ_HD is `static inline` in host builds)
#if defined(__CUDACC__)
#define CZ_MEM __host__ __device__ __forceinline__
#else
#define CZ_MEM inline
#endif

namespace cz {
namespace zl {

constexpr int kMaxBits = 15;
constexpr int kFastBits = 10;  // codes up to this length decode with one table lookup
constexpr int kFastMask = (1 << kFastBits) - 1;

// RFC 1951 3.2.5: length codes 257..285 (li = code - 257), distance codes 0..29
CZ_HD int len_extra(int li) { return li < 8 || li == 28 ? 0 : (li - 4) >> 2; }
CZ_HD int len_base(int li)
{
    if (li < 8) return 3 + li;
    if (li == 28) return 258;
    return (((li - 8) & 3) + 4 << len_extra(li)) + 3;
}
CZ_HD int dist_extra(int ds) { return ds < 4 ? 0 : (ds - 2) >> 1; }
CZ_HD int dist_base(int ds) { return ds < 4 ? ds + 1 : ((2 + (ds & 1)) << dist_extra(ds)) + 1; }
// RFC 1951 3.2.7: 16,17,18,0,8,7,9,6,10,5,11,4,12,3,13,2,14,1,15 (5 bits each)
CZ_HD int cl_order(int i)
{
    const unsigned long long lo = 16ull | 17ull << 5 | 18ull << 10 | 0ull << 15 | 8ull << 20 | 7ull << 25 |
                                  9ull << 30 | 6ull << 35 | 10ull << 40 | 5ull << 45 | 11ull << 50 | 4ull << 55;
    const unsigned long long hi = 12ull | 3ull << 5 | 13ull << 10 | 2ull << 15 | 14ull << 20 | 1ull << 25 | 15ull << 30;
    return i < 12 ? (int)((lo >> (5 * i)) & 31) : (int)((hi >> (5 * (i - 12))) & 31);
}

struct Bits {
    const uint8_t *p;
    long long pos, end;  // byte position of the next refill, input size
    unsigned long long buf;
    int cnt;
    bool over;  // bits past the end of the input were consumed
    CZ_MEM void init(const uint8_t *src, long long n)
    {
        p = src;
        pos = 0;
        end = n;
        buf = 0;
        cnt = 0;
        over = false;
    }
    // refills to at least 57 bits (zeros past the end; reading ahead is not
    // consuming). On the GPU, away from the end of the input, whole bytes
    // come from three aligned 32-bit loads.
    CZ_MEM void fill()
    {
#if defined(__CUDA_ARCH__)
        if (pos + 12 <= end) {
            const uintptr_t a = reinterpret_cast<uintptr_t>(p + pos);
            const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
            const unsigned sh = (unsigned)(a & 3) * 8;
            const unsigned long long lo = (unsigned long long)w[1] << 32 | w[0];
            const unsigned long long v = sh ? (lo >> sh) | ((unsigned long long)w[2] << (64 - sh)) : lo;
            const int nbytes = (64 - cnt) >> 3;
            buf |= (nbytes == 8 ? v : (v & ((1ull << (8 * nbytes)) - 1))) << cnt;
            pos += nbytes;
            cnt += 8 * nbytes;
            return;
        }
#endif
        while (cnt <= 56) {
            const unsigned long long b = pos < end ? p[pos] : 0ull;
            ++pos;
            buf |= b << cnt;
            cnt += 8;
        }
    }
    CZ_MEM unsigned get(int n)
    {
        if (n == 0) return 0;
        if (cnt < n) fill();
        const unsigned v = (unsigned)(buf & ((1ull << n) - 1));
        buf >>= n;
        cnt -= n;
        if (8 * pos - cnt > 8 * end) over = true;
        return v;
    }
    CZ_MEM void align()
    {
        const int drop = cnt & 7;
        buf >>= drop;
        cnt -= drop;
    }
};

// Canonical code: count[len] codes of each length, symbols sorted by code,
// and a table of the codes up to kFastBits long, indexed by the next
// kFastBits input bits: length << 9 | symbol (0: a longer code).
struct Huff {
    unsigned short count[kMaxBits + 1];
    unsigned short sym[288];
    unsigned short fast[1 << kFastBits];
};

// Builds the code from lengths. Rejected as zlib rejects them: oversubscribed
// sets, and incomplete sets except an empty one or a single code of length
// 1 (the code-length code must be complete).
CZ_HD bool build(Huff &h, const unsigned char *len, int n, bool codelen)
{
    for (int i = 0; i <= kMaxBits; ++i) h.count[i] = 0;
    for (int s = 0; s < n; ++s) h.count[len[s]]++;
    h.count[0] = 0;
    int left = 1, maxlen = 0;
    for (int i = 1; i <= kMaxBits; ++i) {
        left <<= 1;
        left -= h.count[i];
        if (left < 0) return false;
        if (h.count[i]) maxlen = i;
    }
    if (left > 0 && maxlen > 0 && (codelen || maxlen != 1)) return false;
    unsigned short offs[kMaxBits + 1];
    offs[1] = 0;
    for (int i = 1; i < kMaxBits; ++i) offs[i + 1] = offs[i] + h.count[i];
    for (int s = 0; s < n; ++s)
        if (len[s]) h.sym[offs[len[s]]++] = (unsigned short)s;
    // lookup table: canonical codes in symbol order per length, bit-reversed
    // (the stream sends codes most significant bit first)
    for (int i = 0; i <= kFastMask; ++i) h.fast[i] = 0;
    int next[kFastBits + 1], code = 0;
    next[0] = 0;
    for (int l = 1; l <= kFastBits; ++l) {
        code = (code + h.count[l - 1]) << 1;
        next[l] = code;
    }
    for (int s = 0; s < n; ++s) {
        const int l = len[s];
        if (!l || l > kFastBits) continue;
        unsigned v = (unsigned)next[l]++, r = 0;
        for (int k = 0; k < l; ++k) {
            r = (r << 1) | (v & 1u);
            v >>= 1;
        }
        for (unsigned i = r; i <= (unsigned)kFastMask; i += 1u << l) h.fast[i] = (unsigned short)(l << 9 | s);
    }
    return true;
}

// Next symbol (codes are read most significant bit first), -1 on error:
// one table lookup for codes up to kFastBits, the canonical walk (one bit
// per length) otherwise.
CZ_HD int decode_slow(Bits &b, const Huff &h)
{
    int code = 0, first = 0, index = 0;
    for (int len = 1; len <= kMaxBits; ++len) {
        code |= (int)b.get(1);
        const int count = h.count[len];
        if (code - count < first) return h.sym[index + (code - first)];
        index += count;
        first += count;
        first <<= 1;
        code <<= 1;
    }
    return -1;
}
CZ_HD int decode(Bits &b, const Huff &h)
{
    if (b.cnt < kFastBits) b.fill();
    const unsigned e = h.fast[b.buf & kFastMask];
    if (!e) return decode_slow(b, h);
    const int l = (int)(e >> 9);
    b.buf >>= l;
    b.cnt -= l;
    if (8 * b.pos - b.cnt > 8 * b.end) b.over = true;
    return (int)(e & 511);
}

// Decoder state across batches.
struct Inflater {
    Bits b;
    long long op;  // output written so far (literals, recorded matches and runs)
    int err, final_block, in_block, btype;
    long long stored_left;
    // a stored block's bytes, for the caller to copy: input position,
    // output position, length (run_n = 0: none)
    long long run_src, run_dst, run_n;

    // Reads the zlib header; err != 0 if it is not a deflate stream without
    // a preset dictionary (RFC 1950 2.2).
    CZ_MEM void start(const uint8_t *src, long long n)
    {
        b.init(src, n);
        op = 0;
        err = final_block = in_block = btype = 0;
        stored_left = 0;
        run_src = run_dst = run_n = 0;
        const unsigned cmf = b.get(8), flg = b.get(8);
        if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 || (flg & 32)) err = 1;
    }

    // Reads a block header at the current position (BFINAL, BTYPE; LEN/NLEN
    // of a stored block; the code tables of a Huffman block, built into lit
    // and dist). Returns err (0: the block's data follows).
    CZ_MEM int block_header(Huff &lit, Huff &dist, unsigned char *lens)
    {
        final_block = (int)b.get(1);
        btype = (int)b.get(2);
        in_block = 1;
        if (btype == 0) {
            b.align();
            const unsigned l = b.get(16), nl = b.get(16);
            if ((l ^ 0xffffu) != nl || b.over) return err = 2;
            stored_left = l;
        } else if (btype == 1) {
            for (int i = 0; i < 288; ++i) lens[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
            build(lit, lens, 288, false);
            // all 32 fixed distance codes (30 and 31 never occur, RFC 1951 3.2.6)
            for (int i = 0; i < 32; ++i) lens[i] = 5;
            build(dist, lens, 32, false);
        } else if (btype == 2) {
            const int nlen = (int)b.get(5) + 257, ndist = (int)b.get(5) + 1, ncode = (int)b.get(4) + 4;
            if (nlen > 286 || ndist > 30) return err = 3;
            for (int i = 0; i < 19; ++i) lens[i] = 0;
            for (int i = 0; i < ncode; ++i) lens[cl_order(i)] = (unsigned char)b.get(3);
            if (!build(lit, lens, 19, true)) return err = 4;
            int i = 0;
            while (i < nlen + ndist) {
                const int sym = decode(b, lit);
                if (sym < 0 || b.over) return err = 5;
                if (sym < 16) {
                    lens[i++] = (unsigned char)sym;
                    continue;
                }
                int rep = 0, val = 0;
                if (sym == 16) {
                    if (i == 0) return err = 6;
                    val = lens[i - 1];
                    rep = 3 + (int)b.get(2);
                } else if (sym == 17) {
                    rep = 3 + (int)b.get(3);
                } else {
                    rep = 11 + (int)b.get(7);
                }
                if (i + rep > nlen + ndist) return err = 7;
                while (rep--) lens[i++] = (unsigned char)val;
            }
            if (lens[256] == 0) return err = 8;
            if (!build(lit, lens, nlen, false)) return err = 9;
            if (!build(dist, lens + nlen, ndist, false)) return err = 10;
        } else {
            return err = 11;
        }
        return 0;
    }

    // Decodes until `cap` matches are recorded (batch[i] = {position,
    // length, distance}), a stored block's bytes are reached, the last block
    // ends, or an error. Literals go to dst directly; matches are for the
    // caller to copy in order, and so is a stored block (run_src, run_dst,
    // run_n: input to output, disjoint from the matches). Returns the number
    // of matches recorded.
    CZ_MEM int step(uint8_t *dst, long long oend, int (*batch)[3], int cap, Huff &lit, Huff &dist,
                   unsigned char *lens)
    {
        int n = 0;
        run_n = 0;
        while (!err && n < cap) {
            if (!in_block) {
                if (final_block) break;
                if (block_header(lit, dist, lens)) break;
            }
            if (btype == 0) {  // stored bytes (byte aligned): one run for the caller
                const long long from = b.pos - b.cnt / 8;  // next unread input byte (cnt is whole bytes here)
                if (op + stored_left > oend) {
                    err = 12;
                    break;
                }
                if (from + stored_left > b.end) {
                    err = 13;
                    break;
                }
                run_src = from;
                run_dst = op;
                run_n = stored_left;
                op += stored_left;
                b.pos = from + stored_left;
                b.buf = 0;
                b.cnt = 0;
                stored_left = 0;
                in_block = 0;
                break;  // copied before the next step
            }
            // literals while at least 8 input and 8 output bytes remain: one
            // table lookup each and no per-symbol end tests (a refill then
            // stays within the input, a literal within the output); other
            // symbols and long codes take the general path below
            {
                const long long olim = oend - 8, ilim = b.end - 8;
                while (op <= olim && b.pos <= ilim) {
                    if (b.cnt < kFastBits) b.fill();
                    const unsigned e = lit.fast[b.buf & kFastMask];
                    if (!e || (e & 511u) >= 256u) break;
                    const int l = (int)(e >> 9);
                    b.buf >>= l;
                    b.cnt -= l;
                    dst[op++] = (uint8_t)e;
                }
            }
            const int sym = decode(b, lit);
            if (sym < 0 || b.over) {
                err = 14;
                break;
            }
            if (sym < 256) {
                if (op >= oend) {
                    err = 15;
                    break;
                }
                dst[op++] = (uint8_t)sym;
            } else if (sym == 256) {
                in_block = 0;
            } else {
                const int li = sym - 257;
                if (li >= 29) {
                    err = 16;
                    break;
                }
                const int len = len_base(li) + (int)b.get(len_extra(li));
                const int ds = decode(b, dist);
                if (ds < 0 || ds >= 30) {
                    err = 17;
                    break;
                }
                const int d = dist_base(ds) + (int)b.get(dist_extra(ds));
                if (b.over) {
                    err = 18;
                    break;
                }
                if (d > op) {
                    err = 19;
                    break;
                }
                if (op + len > oend) {
                    err = 20;
                    break;
                }
                batch[n][0] = (int)op;
                batch[n][1] = len;
                batch[n][2] = d;
                ++n;
                op += len;
            }
        }
        return n;
    }

    CZ_MEM bool done() const { return !in_block && final_block; }

    // After the last block: the big-endian Adler-32 (RFC 1950 2.2); err set
    // if it is missing.
    CZ_MEM unsigned trailer()
    {
        b.align();
        const unsigned t3 = b.get(8), t2 = b.get(8), t1 = b.get(8), t0 = b.get(8);
        if (b.over) err = 21;
        return (t3 << 24) | (t2 << 16) | (t1 << 8) | t0;
    }
};

}  // namespace zl
}  // namespace cz
