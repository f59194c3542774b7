// cz_deflate_emu.cpp -- host build of the GPU zlib encoder's serial part
// (cz_deflate.cuh): the same blocks, symbol counts, code construction,
// per-block coding choice and symbol emission as the kernel, done serially,
// plus a small greedy LZ77 parse to feed it, so the CPU suite can decode the
// streams with zlib and check every block's counted size. Test
// infrastructure only.
#include <string.h>

#include <vector>

#include "../../cubismz_gb300/csrc/cz_deflate.cuh"

using namespace cz::zl;

namespace {

struct BitW {
    uint8_t *o;
    long long cap, bp;
    bool over;
    void put(unsigned long long v, int n)
    {
        for (int i = 0; i < n; ++i, ++bp) {
            const long long byte = bp >> 3;
            if (byte >= cap) {
                over = true;
                continue;
            }
            if ((v >> i) & 1ull) o[byte] |= (uint8_t)(1u << (bp & 7));
        }
    }
};

// lengths for the used symbols of freq[0..n) (at least two, dummies of
// weight one added), sorted by (frequency, symbol) like the kernel
bool build(const uint32_t *freq, int n, int maxbits, uint8_t *len)
{
    std::vector<int> sym;
    std::vector<uint32_t> wt(n);
    for (int s = 0; s < n; ++s) {
        wt[s] = freq[s];
        if (freq[s]) sym.push_back(s);
    }
    for (int s = 0; sym.size() < 2 && s < n; ++s)
        if (!freq[s]) {
            wt[s] = 1;
            sym.push_back(s);
        }
    for (size_t a = 1; a < sym.size(); ++a) {
        const int t = sym[a];
        size_t b = a;
        while (b > 0 && (wt[sym[b - 1]] > wt[t] || (wt[sym[b - 1]] == wt[t] && sym[b - 1] > t))) {
            sym[b] = sym[b - 1];
            --b;
        }
        sym[b] = t;
    }
    const int m = (int)sym.size();
    std::vector<uint32_t> w(m), iw(m);
    std::vector<uint16_t> par(2 * m), dep(2 * m);
    std::vector<uint8_t> l(m);
    for (int i = 0; i < m; ++i) w[i] = wt[sym[i]];
    if (!huff_lengths(w.data(), m, maxbits, l.data(), iw.data(), par.data(), dep.data())) return false;
    for (int s = 0; s < n; ++s) len[s] = 0;
    for (int i = 0; i < m; ++i) len[sym[i]] = l[i];
    return true;
}

}  // namespace

// Greedy parse with one candidate per 4-byte hash; matches of 4 bytes or
// more, distances up to max_dist, lengths up to max_len. Records as the GPU
// parse writes them; the last one carries the tail literals.
extern "C" int emu_parse(const uint8_t *src, int L, int max_dist, int max_len, unsigned long long *seq, int cap)
{
    std::vector<int> table(1 << 15, -1);
    int p = 0, anchor = 0, n = 0;
    while (p + 4 <= L) {
        uint32_t v;
        memcpy(&v, src + p, 4);
        const uint32_t h = (v * 2654435761u) >> 17;
        const int c = table[h];
        table[h] = p;
        if (c >= 0 && p - c <= max_dist && memcmp(src + c, src + p, 4) == 0) {
            int m = 4;
            while (p + m < L && m < max_len && src[c + m] == src[p + m]) ++m;
            if (n >= cap) return -1;
            seq[n++] = seq_pack(p - anchor, m, p - c);
            p += m;
            anchor = p;
        } else {
            ++p;
        }
    }
    if (n >= cap) return -1;
    seq[n++] = seq_pack(L - anchor, 0, 0);
    return n;
}

// zlib stream of src[0..L) from its parse, with the kernel's blocks (one
// per mask / byte plane of each record when `records`, else per 65535
// bytes) and per-block choice. mode: -1 smallest per block, 0 stored,
// 1 fixed, 2 dynamic (forced where allowed). Returns the stream size, -1 on
// a bad parse, -2 when a block's written bits differ from its count.
extern "C" long long emu_deflate(const uint8_t *src, int L, const unsigned long long *seq, int nseq, int mode,
                                 int records, uint8_t *out, long long cap, long long *nblocks)
{
    // item list: (position, literal byte or -(piece length), distance)
    struct Item {
        int pos, v, d;
    };
    std::vector<Item> items;
    long long pos = 0;
    for (int i = 0; i < nseq; ++i) {
        const int lit = seq_lit(seq[i]), m = seq_mlen(seq[i]), d = seq_dist(seq[i]);
        if (pos + lit + m > L) return -1;
        for (int k = 0; k < lit; ++k) items.push_back({(int)(pos + k), src[pos + k], 0});
        pos += lit;
        if (m) {
            if (d < 1 || d > kMaxDist || d > pos || m < 3) return -1;
            for (int k = 0; k < npieces(m); ++k) {
                if (piece_start(m, k) != (k ? piece_start(m, k - 1) + piece_len(m, k - 1) : 0)) return -1;
                if (pieces_before(m, piece_start(m, k)) != k || pieces_before(m, piece_start(m, k) + 1) != k + 1)
                    return -1;
                items.push_back({(int)(pos + piece_start(m, k)), -piece_len(m, k), d});
            }
            pos += m;
        }
    }
    if (pos != L) return -1;
    memset(out, 0, (size_t)cap);
    out[0] = 0x78;
    out[1] = 0x9c;
    BitW w{out, cap, 16, false};
    Bounds bnd;
    bnd.init(src, L, records != 0);
    size_t it = 0;
    int lo = 0;
    *nblocks = 0;
    static Codes dyn, fix;
    fixed_codes(fix);
    for (;;) {
        const int hi = bnd.next(lo);
        uint32_t lf[288] = {0}, df[32] = {0};
        lf[256] = 1;
        size_t e = it;
        int cov = lo;
        for (; e < items.size() && items[e].pos < hi; ++e) {
            const Item &x = items[e];
            if (x.v >= 0) {
                lf[x.v]++;
                cov = x.pos + 1;
            } else {
                lf[257 + len_sym(-x.v)]++;
                df[dist_sym(x.d)]++;
                cov = x.pos - x.v;
            }
        }
        const bool final = cov >= L;
        memset(&dyn, 0, sizeof dyn);
        long long dbits = -1;
        if (build(lf, kLitSyms, kMaxLit, dyn.llen) && build(df, kDistSyms, kMaxLit, dyn.dlen)) {
            canon_codes(dyn.llen, 288, dyn.lcode);
            canon_codes(dyn.dlen, 32, dyn.dcode);
            const long long hb = dynamic_header(dyn);
            if (hb >= 0) dbits = hb + data_bits(lf, df, dyn.llen, dyn.dlen);
        }
        const long long fbits = fixed_block_bits(lf, df);
        const long long sbits = cov - lo <= kStoredMax ? stored_block_bits(w.bp, cov - lo) : -1;
        int md = 2;
        long long best = dbits;
        if (dbits < 0 || fbits <= dbits) {
            md = 1;
            best = fbits;
        }
        if (sbits >= 0 && sbits <= best) {
            md = 0;
            best = sbits;
        }
        if (mode == 0 && sbits >= 0) md = 0, best = sbits;
        if (mode == 1) md = 1, best = fbits;
        if (mode == 2 && dbits >= 0) md = 2, best = dbits;
        const long long bp0 = w.bp;
        if (md == 0) {
            w.put(final ? 1u : 0u, 3);
            w.bp = (w.bp + 7) & ~7ll;
            const unsigned n = (unsigned)(cov - lo);
            w.put(n | (~n & 0xffffu) << 16, 32);
            for (int k = lo; k < cov; ++k) w.put(src[k], 8);
        } else {
            const Codes &c = md == 1 ? fix : dyn;
            if (md == 1) w.put((final ? 1u : 0u) | 1u << 1, 3);
            else put_dynamic_header(w, c, final);
            for (size_t k = it; k < e; ++k) {
                const Item &x = items[k];
                if (x.v >= 0) {
                    w.put(c.lcode[x.v], c.llen[x.v]);
                } else {
                    unsigned long long v;
                    const int nb = match_bits(c, -x.v, x.d, v);
                    w.put(v, nb);
                }
            }
            w.put(c.lcode[256], c.llen[256]);
        }
        if (w.bp - bp0 != best) return -2;
        ++*nblocks;
        it = e;
        if (final) break;
        if (cov <= lo) return -3;
        lo = cov;
    }
    if (w.over) return -1;
    long long op = (w.bp + 7) >> 3;
    unsigned long long a = 1, b = 0;
    for (int i = 0; i < L; ++i) {
        a = (a + src[i]) % 65521;
        b = (b + a) % 65521;
    }
    const unsigned ad = (unsigned)((b << 16) | a);
    if (op + 4 > cap) return -1;
    out[op++] = (uint8_t)(ad >> 24);
    out[op++] = (uint8_t)(ad >> 16);
    out[op++] = (uint8_t)(ad >> 8);
    out[op++] = (uint8_t)ad;
    return op;
}

// huff_lengths alone: lengths for weights sorted ascending.
extern "C" int emu_huff_lengths(const uint32_t *w, int n, int maxbits, uint8_t *len)
{
    std::vector<uint32_t> iw(n);
    std::vector<uint16_t> par(2 * n), dep(2 * n);
    return huff_lengths(w, n, maxbits, len, iw.data(), par.data(), dep.data()) ? 1 : 0;
}
