// cz_zlib.cu -- zlib streams (RFC 1950 wrapper, RFC 1951 DEFLATE), the
// format of the reference's zlib encoder (deflateInit/deflate with Z_FINISH,
// CompressionEncoders.h:116-190) and decoder (inflateInit/inflate,
// CompressionEncoders.h:48-88).
//
// Decoder: one warp per chunk. Lane 0 reads the header and the blocks
// (stored, fixed Huffman, dynamic Huffman) and decodes symbols with the
// canonical codes (per code length: count and first symbol, so a symbol
// costs one bit test per code length); it records a batch of sequences
// (literal run from the output it wrote, match length, distance). The warp
// then copies the batch's matches in order, each byte-parallel: byte k of a
// match at p with distance d is out[p - d + (k mod d)], always already
// written. The Adler-32 of the output is a warp reduction, checked against
// the trailer. Malformed input (bad header, code lengths, symbols,
// distances past the start, output past the capacity, truncated input or a
// wrong checksum) gives a negative length; every read and write is bounds
// checked.
#include "cz_codec.h"
#include "cz_inflate.cuh"

namespace cz {

using namespace zl;

constexpr int kZBatch = 128;  // matches per batch

__global__ void __launch_bounds__(32)
inflate_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
               uint8_t *__restrict__ out, const long long *out_off, const int *out_cap, int *out_len)
{
    __shared__ Huff lit, dist;
    __shared__ unsigned char lens[320];
    __shared__ int batch[kZBatch][3];  // matches: output position, length, distance
    __shared__ int s_state[4];         // matches in the batch, error, done, Adler-32 of the trailer
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
            }
            __syncwarp();
            // the warp replays the matches in order, each byte-parallel:
            // byte k of a match at p with distance d is out[p - d + (k mod d)]
            const int n = s_state[0];
            for (int i = 0; i < n; ++i) {
                const int p = batch[i][0], len = batch[i][1], d = batch[i][2];
                for (int k = lane; k < len; k += 32) dst[p + k] = __ldcg(dst + p - d + (d >= len ? k : k % d));
                __syncwarp();
            }
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

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_inflate(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks, uint8_t *out,
                              const long long *out_off, const int *out_cap, int *out_len, int grid, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    inflate_kernel<<<grid, 32, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_cap, out_len);
    return cudaGetLastError();
}
