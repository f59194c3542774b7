// cz_inflate_emu.cpp -- host build of the GPU zlib decoder's serial part
// (cz_inflate.cuh), with the match replay and the Adler-32 check done
// serially, so the CPU test suite can compare it with zlib. Test
// infrastructure only.
#include "../../cubismz_gb300/csrc/cz_inflate.cuh"

using namespace cz::zl;

extern "C" long long emu_inflate(const uint8_t *src, long long n, uint8_t *dst, long long cap)
{
    static Huff lit, dist;
    static unsigned char lens[320];
    static int batch[128][3];
    Inflater z;
    z.start(src, n);
    for (;;) {
        const int m = z.step(dst, cap, batch, 128, lit, dist, lens);
        if (!z.err && z.run_n > 0) memcpy(dst + z.run_dst, src + z.run_src, (size_t)z.run_n);
        for (int i = 0; i < m; ++i)
            for (int k = 0; k < batch[i][1]; ++k) {
                const int p = batch[i][0], d = batch[i][2];
                dst[p + k] = dst[p - d + (d >= batch[i][1] ? k : k % d)];
            }
        if (z.err || z.done()) break;
    }
    if (z.err) return -z.err;
    const unsigned want = z.trailer();
    if (z.err) return -z.err;
    unsigned long long a = 1, b = 0;
    for (long long i = 0; i < z.op; ++i) {
        a = (a + dst[i]) % 65521;
        b = (b + a) % 65521;
    }
    if (((b << 16) | a) != want) return -22;
    return z.op;
}

