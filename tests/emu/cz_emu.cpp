// cz_emu.cpp -- host build of the kernels' per-line arithmetic and index maps.
//
// Compiles the same headers the CUDA kernels use (cz_line.cuh, cz_layout.cuh)
// for the CPU, so the CPU test suite can check the kernels' exact binary32
// evaluation and their layout maps against the oracle bit for bit without a
// GPU. Test infrastructure only; the product never calls it.
#include "../../cubismz_gb300/csrc/cz_layout.cuh"
#include "../../cubismz_gb300/csrc/cz_line.cuh"

#include <stdint.h>
#include <string.h>

using namespace cz;

static inline int IDX(int x, int y, int z) { return x + 32 * (y + 32 * z); }

// axis 0 = x, 1 = y, 2 = z; lines of length N inside the [0,N)^3 corner
template <int N>
static void pass(float *b, int axis, int fwd, int wtype, long long *stats)
{
    for (int a = 0; a < N; ++a)
        for (int c = 0; c < N; ++c) {
            float line[N];
            int idx[N];
            for (int j = 0; j < N; ++j) {
                int x, y, z;
                if (axis == 0) { x = j; y = a; z = c; }
                else if (axis == 1) { x = a; y = j; z = c; }
                else { x = a; y = c; z = j; }
                idx[j] = IDX(x, y, z);
                line[j] = b[idx[j]];
            }
            if (stats) {
                // classify the line the way the kernels do: sources of the
                // stencils are the even samples (interp forward), the
                // scalings (everything else)
                constexpr int H = N / 2;
                float src[H], h[H], l[H];
                uint32_t amax;
                for (int i = 0; i < H; ++i) {
                    if (wtype == 1 || wtype == 2) src[i] = fwd ? line[2 * i] : line[i];
                    else src[i] = fwd ? CZ_MUL(0.5f, CZ_ADD(line[2 * i], line[2 * i + 1])) : line[i];
                }
                stats[0] += 1;
                if (!line_split<H>(src, h, l, amax)) {
                    stats[1] += 1;
                    for (int i = 0; i + 3 < H; ++i) {
                        const float v[4] = {src[i], src[i + 1], src[i + 2], src[i + 3]};
                        stats[2] += !within<4>(v, max_bits<4>(v), kSpread);
                    }
                }
            }
            if (fwd) fwd_line<N>(line, wtype);
            else inv_line<N>(line, wtype);
            for (int j = 0; j < N; ++j) b[idx[j]] = line[j];
        }
}

extern "C" {

// Forward transform in the kernels' layout (physical = mathematical indices).
void emu_fwt(float *b, int wtype, long long *stats)
{
    pass<32>(b, 0, 1, wtype, stats);
    pass<32>(b, 1, 1, wtype, stats);
    pass<32>(b, 2, 1, wtype, stats);
    pass<16>(b, 2, 1, wtype, stats);
    pass<16>(b, 0, 1, wtype, stats);
    pass<16>(b, 1, 1, wtype, stats);
    pass<8>(b, 1, 1, wtype, stats);
    pass<8>(b, 2, 1, wtype, stats);
    pass<8>(b, 0, 1, wtype, stats);
}

void emu_iwt(float *b, int wtype, long long *stats)
{
    pass<8>(b, 0, 0, wtype, stats);
    pass<8>(b, 2, 0, wtype, stats);
    pass<8>(b, 1, 0, wtype, stats);
    pass<16>(b, 1, 0, wtype, stats);
    pass<16>(b, 0, 0, wtype, stats);
    pass<16>(b, 2, 0, wtype, stats);
    pass<32>(b, 2, 0, wtype, stats);
    pass<32>(b, 1, 0, wtype, stats);
    pass<32>(b, 0, 0, wtype, stats);
}

// Reorder a physical-layout block into the reference's positional layout.
void emu_to_positional(const float *phys, float *pos)
{
    for (int pz = 0; pz < 32; ++pz)
        for (int py = 0; py < 32; ++py)
            for (int px = 0; px < 32; ++px) {
                int x, y, z;
                phys_of_pos(px, py, pz, x, y, z);
                pos[IDX(px, py, pz)] = phys[IDX(x, y, z)];
            }
}

int emu_check_maps(void)
{
    int bad = 0;
    for (int s = 0; s < 32768; ++s) {
        int px, py, pz, x, y, z;
        pos_of_stream(s, px, py, pz);
        if (stream_of_pos(px, py, pz) != s) bad++;
        phys_of_pos(px, py, pz, x, y, z);
        if (mask_index(x, y, z) != IDX(px, py, pz)) bad++;
    }
    return bad;
}

// Whole record codec with the kernels' algorithm (stream-order thresholding).
int emu_block_compress(const float *in, float eps, int wtype, int zerobits, int shuffle, uint8_t *out, int *nbytes)
{
    static float b[32768];
    memcpy(b, in, sizeof(b));
    emu_fwt(b, wtype, 0);
    memset(out, 0, 4096);
    uint32_t *pay = (uint32_t *)(out + 4096);
    int n = 0;
    const uint32_t keepmask = zerobits > 0 ? ~((1u << zerobits) - 1u) : 0xffffffffu;
    for (int s = 0; s < 32768; ++s) {
        int px, py, pz, x, y, z;
        pos_of_stream(s, px, py, pz);
        phys_of_pos(px, py, pz, x, y, z);
        const float v = b[IDX(x, y, z)];
        const bool keep = s < 64 || fabsf(v) > eps;
        if (keep) {
            const int p = IDX(px, py, pz);
            out[p >> 3] |= (uint8_t)(1u << (p & 7));
            uint32_t u;
            memcpy(&u, &v, 4);
            pay[n++] = u & keepmask;
        }
    }
    if (shuffle) {
        static uint8_t t[4 * 32768];
        const uint8_t *src = (const uint8_t *)pay;
        for (int i = 0; i < n; ++i)
            for (int p = 0; p < 4; ++p) t[p * n + i] = src[4 * i + p];
        memcpy(pay, t, 4 * n);
    }
    *nbytes = 4096 + 4 * n;
    return 0;
}

int emu_block_decompress(const uint8_t *in, int nbytes, int wtype, int shuffle, float *out)
{
    static uint32_t pay[32768 + 1];
    int expected = 0;
    for (int i = 0; i < 4096; ++i) expected += __builtin_popcount(in[i]);
    const int nb = nbytes - 4096;
    int nel = nb / 4;
    if (nel - expected == 1) nel--;
    if (nel != expected) return -1;
    if (shuffle) {
        const int c = nb / 4;
        uint8_t *dst = (uint8_t *)pay;
        for (int i = 0; i < c; ++i)
            for (int p = 0; p < 4; ++p) dst[4 * i + p] = in[4096 + i + p * c];
    } else {
        memcpy(pay, in + 4096, 4 * nel);
    }
    int k = 0;
    for (int s = 0; s < 32768; ++s) {
        int px, py, pz, x, y, z;
        pos_of_stream(s, px, py, pz);
        phys_of_pos(px, py, pz, x, y, z);
        const int p = IDX(px, py, pz);
        const bool eat = (in[p >> 3] >> (p & 7)) & 1;
        if (s < 64 && !eat) return -2;
        float v = 0.f;
        if (eat) memcpy(&v, &pay[k++], 4);
        out[IDX(x, y, z)] = v;
    }
    emu_iwt(out, wtype, 0);
    return 0;
}

}
