// cz_deflate.cuh -- the serial parts of DEFLATE encoding (RFC 1951), shared
// by the GPU encoder (cz_zlib.cu, run by one lane per chunk) and the host
// test harness: symbol mapping of lengths and distances, Huffman code
// lengths limited to a maximum length, canonical codes, the run-length
// coding of the code lengths, the dynamic block header and the exact size of
// a block under each coding.
//
// The reference writes zlib streams with deflateInit(Z_DEFAULT_COMPRESSION)
// and deflate(Z_FINISH) (SerializerIO_WaveletCompression_MPI_Simple.h:122,
// CompressionEncoders.h:116-190); any valid stream of the same bytes is read
// by its inflate, so the parse and the codes are this encoder's own.
#pragma once
#include <stdint.h>

#include "cz_inflate.cuh"  // CZ_HD, CZ_MEM, length/distance tables, cl_order

namespace cz {
namespace zl {

constexpr int kLitSyms = 286, kDistSyms = 30, kClSyms = 19;
constexpr int kMaxLit = 15, kMaxCl = 7;
constexpr int kMaxDist = 32768;
constexpr int kStoredMax = 65535;

CZ_HD int ilog2u(unsigned v)
{
#if defined(__CUDA_ARCH__)
    return 31 - __clz((int)v);
#else
    return 31 - __builtin_clz(v);
#endif
}

// Match length 3..258 -> li (symbol 257 + li); 258 takes its own code 285.
CZ_HD int len_sym(int len)
{
    const int v = len - 3;
    if (v < 8) return v;
    if (len == 258) return 28;
    const int e = ilog2u((unsigned)v) - 2;
    return 4 * e + (v >> e);
}
// Distance 1..32768 -> distance code 0..29.
CZ_HD int dist_sym(int d)
{
    const int v = d - 1;
    if (v < 4) return v;
    const int e = ilog2u((unsigned)v) - 1;
    return 2 * e + (v >> e);
}

// A match of m >= 3 bytes is sent as pieces of at most 258 bytes, each at
// least 3: whole pieces of 258, then the remainder r = m mod 258; r of 1 or
// 2 borrows from the last whole piece (255 + r, then 3).
CZ_HD int npieces(int m) { return m / 258 + (m % 258 != 0); }
CZ_HD int piece_len(int m, int k)
{
    const int f = m / 258, r = m % 258;
    if (r == 0 || r >= 3) return k < f ? 258 : r;
    if (k < f - 1) return 258;
    return k == f - 1 ? 255 + r : 3;
}
// Offset of piece k from the match start.
CZ_HD int piece_start(int m, int k)
{
    const int r = m % 258;
    return (m > 258 && (r == 1 || r == 2) && k == m / 258) ? m - 3 : 258 * k;
}
// Number of pieces of a match of m bytes that start before offset x.
CZ_HD int pieces_before(int m, int x)
{
    if (x <= 0) return 0;
    const int np = npieces(m), r = m % 258, c = (x + 257) / 258;
    if (m <= 258 || r == 0 || r >= 3) return c < np ? c : np;
    const int f = m / 258;  // pieces 0..f-1 at 258k, the last at m - 3
    return (c < f ? c : f) + (m - 3 < x ? 1 : 0);
}

// Code lengths for n >= 2 weights sorted ascending: the optimal prefix code
// (two-queue construction over the sorted leaves), limited to maxbits. The
// limit works on the count of codes per length: leaves deeper than maxbits
// are put at maxbits, then, while the Kraft sum exceeds one, a code of
// length maxbits is removed and a shorter code of length b becomes two of
// length b+1 -- the number of codes stays, the sum drops by 2^-maxbits. The
// lengths are then handed out longest first to the smallest weights. On
// return len[i] belongs to weight i. Scratch: iw (n-1), par and dep (2n-1).
CZ_HD bool huff_lengths(const uint32_t *w, int n, int maxbits, uint8_t *len, uint32_t *iw, uint16_t *par,
                        uint16_t *dep)
{
    int i = 0, j = 0;  // next leaf, next internal node
    for (int k = 0; k < n - 1; ++k) {
        uint32_t s = 0;
        for (int t = 0; t < 2; ++t) {
            if (i < n && (j >= k || w[i] <= iw[j])) {
                par[i] = (uint16_t)(n + k);
                s += w[i++];
            } else {
                par[n + j] = (uint16_t)(n + k);
                s += iw[j++];
            }
        }
        iw[k] = s;
    }
    const int root = 2 * n - 2;
    dep[root] = 0;
    for (int x = root - 1; x >= 0; --x) dep[x] = (uint16_t)(dep[par[x]] + 1);  // parents come later
    int cnt[16];
    for (int b = 0; b < 16; ++b) cnt[b] = 0;
    for (int x = 0; x < n; ++x) cnt[dep[x] > maxbits ? maxbits : dep[x]]++;
    unsigned kraft = 0;
    for (int b = 1; b <= maxbits; ++b) kraft += (unsigned)cnt[b] << (maxbits - b);
    while (kraft > (1u << maxbits)) {
        int b = maxbits - 1;
        while (b > 0 && cnt[b] == 0) --b;
        if (b == 0 || cnt[maxbits] == 0) return false;
        cnt[maxbits]--;
        cnt[b]--;
        cnt[b + 1] += 2;
        --kraft;
    }
    int x = 0;
    for (int b = maxbits; b >= 1; --b)
        for (int c = 0; c < cnt[b]; ++c) len[x++] = (uint8_t)b;
    return kraft == (1u << maxbits) && x == n;
}

// Canonical codes (RFC 1951 3.2.2) for lengths len[0..n), bit-reversed for
// the LSB-first bit stream.
CZ_HD void canon_codes(const uint8_t *len, int n, uint16_t *code)
{
    int cnt[16], next[16];
    for (int b = 0; b < 16; ++b) cnt[b] = 0;
    for (int s = 0; s < n; ++s) cnt[len[s]]++;
    cnt[0] = 0;
    int c = 0;
    for (int b = 1; b < 16; ++b) {
        c = (c + cnt[b - 1]) << 1;
        next[b] = c;
    }
    for (int s = 0; s < n; ++s) {
        const int l = len[s];
        if (!l) {
            code[s] = 0;
            continue;
        }
        unsigned v = (unsigned)next[l]++;
#if defined(__CUDA_ARCH__)
        code[s] = (uint16_t)(__brev(v) >> (32 - l));
#else
        unsigned r = 0;
        for (int k = 0; k < l; ++k) {
            r = (r << 1) | (v & 1u);
            v >>= 1;
        }
        code[s] = (uint16_t)r;
#endif
    }
}

// The fixed code lengths (RFC 1951 3.2.6).
CZ_HD int fixed_lit_len(int s) { return s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8)); }

// Run-length coding of the code lengths (RFC 1951 3.2.7): entries
// sym | extra << 8 (16: repeat the previous 3-6 times, 17: 3-10 zeros,
// 18: 11-138 zeros). Returns the number of entries (at most n).
CZ_HD int rle_lengths(const uint8_t *L, int n, uint16_t *out)
{
    int m = 0, i = 0;
    while (i < n) {
        const int v = L[i];
        int run = 1;
        while (i + run < n && L[i + run] == v) ++run;
        i += run;
        if (v == 0) {
            while (run >= 11) {
                const int r = run < 138 ? run : 138;
                out[m++] = (uint16_t)(18 | (r - 11) << 8);
                run -= r;
            }
            if (run >= 3) {
                out[m++] = (uint16_t)(17 | (run - 3) << 8);
                run = 0;
            }
        } else {
            out[m++] = (uint16_t)v;
            --run;
            while (run >= 3) {
                const int r = run < 6 ? run : 6;
                out[m++] = (uint16_t)(16 | (r - 3) << 8);
                run -= r;
            }
        }
        while (run-- > 0) out[m++] = (uint16_t)v;
    }
    return m;
}
CZ_HD int rle_extra_bits(int sym) { return sym == 16 ? 2 : (sym == 17 ? 3 : (sym == 18 ? 7 : 0)); }

// The codes of one block.
struct Codes {
    uint8_t llen[288], dlen[32], clen[kClSyms];
    uint16_t lcode[288], dcode[32], ccode[kClSyms];
    uint16_t rle[kLitSyms + kDistSyms];
    int nrle, hlit, hdist, hclen;
};

// Bits of the symbols of a block under the given lengths (end of block
// included in lf): data bits plus the length and distance extra bits.
CZ_HD long long data_bits(const uint32_t *lf, const uint32_t *df, const uint8_t *llen, const uint8_t *dlen)
{
    long long b = 0;
    for (int s = 0; s < kLitSyms; ++s) b += (long long)lf[s] * llen[s];
    for (int li = 0; li < 29; ++li) b += (long long)lf[257 + li] * len_extra(li);
    for (int d = 0; d < kDistSyms; ++d) b += (long long)df[d] * (dlen[d] + dist_extra(d));
    return b;
}

// After llen/dlen are set: hlit, hdist, the run-length entries and the
// code-length code (built serially: 19 symbols). Returns the header bits
// (block type included), or -1 if the code-length code cannot be built.
CZ_HD long long dynamic_header(Codes &c)
{
    int hl = kLitSyms, hd = kDistSyms;
    while (hl > 257 && c.llen[hl - 1] == 0) --hl;
    while (hd > 1 && c.dlen[hd - 1] == 0) --hd;
    c.hlit = hl;
    c.hdist = hd;
    uint8_t all[kLitSyms + kDistSyms];
    for (int s = 0; s < hl; ++s) all[s] = c.llen[s];
    for (int s = 0; s < hd; ++s) all[hl + s] = c.dlen[s];
    c.nrle = rle_lengths(all, hl + hd, c.rle);
    uint32_t cf[kClSyms];
    for (int s = 0; s < kClSyms; ++s) cf[s] = 0;
    for (int i = 0; i < c.nrle; ++i) cf[c.rle[i] & 31]++;
    // symbols by (frequency, symbol), at least two of them
    int sym[kClSyms], m = 0;
    for (int s = 0; s < kClSyms; ++s)
        if (cf[s]) sym[m++] = s;
    for (int s = 0; m < 2 && s < kClSyms; ++s)
        if (!cf[s]) {
            cf[s] = 1;  // never sent; keeps the code complete
            sym[m++] = s;
        }
    for (int a = 1; a < m; ++a) {
        const int t = sym[a];
        int b = a;
        while (b > 0 && (cf[sym[b - 1]] > cf[t] || (cf[sym[b - 1]] == cf[t] && sym[b - 1] > t))) {
            sym[b] = sym[b - 1];
            --b;
        }
        sym[b] = t;
    }
    uint32_t w[kClSyms], iw[kClSyms];
    uint16_t par[2 * kClSyms], dep[2 * kClSyms];
    uint8_t l[kClSyms];
    for (int i = 0; i < m; ++i) w[i] = cf[sym[i]];
    if (!huff_lengths(w, m, kMaxCl, l, iw, par, dep)) return -1;
    for (int s = 0; s < kClSyms; ++s) c.clen[s] = 0;
    for (int i = 0; i < m; ++i) c.clen[sym[i]] = l[i];
    canon_codes(c.clen, kClSyms, c.ccode);
    int hc = kClSyms;
    while (hc > 4 && c.clen[cl_order(hc - 1)] == 0) --hc;
    c.hclen = hc;
    long long bits = 3 + 5 + 5 + 4 + 3 * hc;
    for (int i = 0; i < c.nrle; ++i) {
        const int s = c.rle[i] & 31;
        bits += c.clen[s] + rle_extra_bits(s);
    }
    return bits;
}

// Writes the block header (BFINAL, BTYPE = 2) and the code description.
template <class W>
CZ_HD void put_dynamic_header(W &w, const Codes &c, bool final)
{
    w.put((final ? 1u : 0u) | 2u << 1, 3);
    w.put((unsigned)(c.hlit - 257), 5);
    w.put((unsigned)(c.hdist - 1), 5);
    w.put((unsigned)(c.hclen - 4), 4);
    for (int i = 0; i < c.hclen; ++i) w.put(c.clen[cl_order(i)], 3);
    for (int i = 0; i < c.nrle; ++i) {
        const int s = c.rle[i] & 31, e = c.rle[i] >> 8;
        w.put(c.ccode[s], c.clen[s]);
        if (s >= 16) w.put((unsigned)e, rle_extra_bits(s));
    }
}

// Fixed codes into c (lengths and bit-reversed codes).
CZ_HD void fixed_codes(Codes &c)
{
    for (int s = 0; s < 288; ++s) c.llen[s] = (uint8_t)fixed_lit_len(s);
    for (int d = 0; d < 32; ++d) c.dlen[d] = 5;
    canon_codes(c.llen, 288, c.lcode);
    canon_codes(c.dlen, 32, c.dcode);
}

// Bits of one match piece (length code and extra, distance code and extra)
// and the value to send, LSB first; at most 48 bits.
CZ_HD int match_bits(const Codes &c, int len, int dist, unsigned long long &v)
{
    const int li = len_sym(len), ds = dist_sym(dist);
    const int le = len_extra(li), de = dist_extra(ds);
    int n = 0;
    v = c.lcode[257 + li];
    n = c.llen[257 + li];
    v |= (unsigned long long)(len - len_base(li)) << n;
    n += le;
    v |= (unsigned long long)c.dcode[ds] << n;
    n += c.dlen[ds];
    v |= (unsigned long long)(dist - dist_base(ds)) << n;
    n += de;
    return n;
}

// Bytes of the stored coding of n bytes: one byte of block header and four
// of LEN/NLEN per block of at most 65535 bytes (at least one block).
CZ_HD long long stored_bytes(long long n)
{
    const long long blocks = n == 0 ? 1 : (n + kStoredMax - 1) / kStoredMax;
    return n + 5 * blocks;
}
// Bits of one stored block of n <= 65535 bytes starting at bit position bp:
// header, padding to the byte boundary, LEN/NLEN, the bytes.
CZ_HD long long stored_block_bits(long long bp, int n)
{
    const long long after = bp + 3;
    return 3 + ((8 - (after & 7)) & 7) + 32 + 8ll * n;
}
// Bits of a fixed-code block (header and end of block included in lf).
CZ_HD long long fixed_block_bits(const uint32_t *lf, const uint32_t *df)
{
    long long b = 3;
    for (int x = 0; x < kLitSyms; ++x) b += (long long)lf[x] * fixed_lit_len(x);
    for (int li = 0; li < 29; ++li) b += (long long)lf[257 + li] * len_extra(li);
    for (int d = 0; d < kDistSyms; ++d) b += (long long)df[d] * (5 + dist_extra(d));
    return b;
}

// Block boundaries of a chunk. Chunks of block records with byte-plane
// shuffle ([int32 nbytes][4096-byte mask][S low bytes]...[S high bytes]
// per record) end a block at the mask and at every plane, where the
// statistics change; other chunks every 65535 bytes. Segments shorter
// than kMinBlock merge into the next one.
constexpr int kMinBlock = 1024;
struct Bounds {
    const uint8_t *src;
    int L, rec, k, S;  // current record start, next boundary index in it, its S
    bool records;
    CZ_MEM void init(const uint8_t *s, int n, bool recs)
    {
        src = s;
        L = n;
        rec = 0;
        k = 0;
        S = -1;
        records = recs;
    }
    // boundary k of the record at rec (k = 0..4: mask end, plane ends)
    CZ_MEM int at(int kk) const { return kk == 0 ? rec + 4 + 4096 : rec + 4 + 4096 + kk * S; }
    CZ_MEM bool load_record()
    {
        if (rec + 4 > L) return false;
        const int nb = (int)((unsigned)src[rec] | (unsigned)src[rec + 1] << 8 | (unsigned)src[rec + 2] << 16 |
                             (unsigned)src[rec + 3] << 24);
        if (nb < 4096 || nb > 4096 + 4 * 32768 || (nb - 4096) % 4 || rec + 4 + nb > L) return false;
        S = (nb - 4096) / 4;
        k = 0;
        return true;
    }
    // The first boundary at least kMinBlock past lo (L at most).
    CZ_MEM int next(int lo)
    {
        if (!records) {
            const int b = lo + kStoredMax;
            return b < L ? b : L;
        }
        for (;;) {
            if (S < 0 && !load_record()) return L;
            while (k <= 4) {
                const int b = at(k);
                if (b >= lo + kMinBlock) return b < L ? b : L;
                ++k;
            }
            rec = at(4);  // next record
            S = -1;
        }
    }
};

// Packed parse record: literal run, match length (0: none), distance.
CZ_HD unsigned long long seq_pack(int lit, int mlen, int dist)
{
    return (unsigned long long)(unsigned)lit | (unsigned long long)(unsigned)mlen << 24 |
           (unsigned long long)(unsigned)dist << 48;
}
CZ_HD int seq_lit(unsigned long long r) { return (int)(r & 0xffffffu); }
CZ_HD int seq_mlen(unsigned long long r) { return (int)((r >> 24) & 0xffffffu); }
CZ_HD int seq_dist(unsigned long long r) { return (int)(r >> 48); }

}  // namespace zl
}  // namespace cz
