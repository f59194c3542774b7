// lz4rec_main.cpp -- command-line runner of lz4rec_emu.cpp (a separate
// executable, so that it can be built with AddressSanitizer):
//   lz4rec_emu <dir>   reads <dir>/meta.bin and <dir>/in.bin, writes
//                      <dir>/out.bin (the LZ4 blocks back to back) and
//                      <dir>/off.bin (nchunks + 1 offsets).
// meta.bin: int32 nchunks, bpc, shuffle, ctas, seed, has_blk_dst; int64
// nblocks; int64 in_off[nchunks]; int32 in_len[nchunks]; int32
// rec_bytes[nblocks]; int64 blk_dst[nblocks] when has_blk_dst.
#include "lz4rec_emu.cpp"

#include <string>

static std::vector<char> slurp(const std::string &p)
{
    FILE *f = fopen(p.c_str(), "rb");
    if (!f) exit(2);
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> v((size_t)n);
    if (n && fread(v.data(), 1, (size_t)n, f) != (size_t)n) exit(2);
    fclose(f);
    return v;
}

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    const std::vector<char> meta = slurp(dir + "/meta.bin"), inb = slurp(dir + "/in.bin");
    const char *m = meta.data();
    int hdr[6];
    memcpy(hdr, m, sizeof hdr);
    m += sizeof hdr;
    long long nblocks;
    memcpy(&nblocks, m, 8);
    m += 8;
    const int n = hdr[0], bpc = hdr[1], shuffle = hdr[2], ctas = hdr[3], has_dst = hdr[5];
    const unsigned seed = (unsigned)hdr[4];
    std::vector<long long> in_off(n), blk_dst(has_dst ? nblocks : 0), lz_off(n), dst_off(n + 1);
    std::vector<int> in_len(n), rec((size_t)nblocks), out_len(n);
    memcpy(in_off.data(), m, 8 * (size_t)n);
    m += 8 * (size_t)n;
    memcpy(in_len.data(), m, 4 * (size_t)n);
    m += 4 * (size_t)n;
    memcpy(rec.data(), m, 4 * (size_t)nblocks);
    m += 4 * (size_t)nblocks;
    if (has_dst) memcpy(blk_dst.data(), m, 8 * (size_t)nblocks);
    // exact-size buffers: the input with the 4 bytes of tail room the
    // kernels may read, the region slots, the output
    uint8_t *in = static_cast<uint8_t *>(malloc(inb.size() + 4));
    memcpy(in, inb.data(), inb.size());
    memset(in + inb.size(), 0, 4);
    long long mx = 0, total = 0;
    for (int c = 0; c < n; ++c) mx = std::max<long long>(mx, in_len[c]);
    const long long slot = ((mx + (mx >> 3) + 64LL * 3 * bpc + 64) + 15) / 16 * 16;
    for (int c = 0; c < n; ++c) lz_off[c] = slot * c;
    uint8_t *lz = static_cast<uint8_t *>(malloc((size_t)(slot * n)));
    LzRegion *reg = static_cast<LzRegion *>(malloc(sizeof(LzRegion) * 3 * (size_t)bpc * n));
    for (int c = 0; c < n; ++c) total += in_len[c] + in_len[c] / 8 + 64;
    uint8_t *out = static_cast<uint8_t *>(malloc((size_t)total));
    const int rc = emu_lz4rec(in, in_off.data(), in_len.data(), n, rec.data(), has_dst ? blk_dst.data() : nullptr,
                              nblocks, bpc, shuffle, lz, lz_off.data(), reg, out_len.data(), out, dst_off.data(), ctas,
                              seed);
    if (rc != 0) return 3;
    FILE *f = fopen((dir + "/out.bin").c_str(), "wb");
    fwrite(out, 1, (size_t)dst_off[n], f);
    fclose(f);
    f = fopen((dir + "/off.bin").c_str(), "wb");
    fwrite(dst_off.data(), 8, (size_t)n + 1, f);
    fclose(f);
    free(in);
    free(lz);
    free(reg);
    free(out);
    return 0;
}
