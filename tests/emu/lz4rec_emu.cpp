// lz4rec_emu.cpp -- host build of the region-parallel LZ4 kernels
// (cubismz_gb300/csrc/cz_lz4rec.cu) on the warp emulator of warp_emu.h.
//
// tests/test_lz4rec_emu.py writes the kernel source, without its includes,
// to lz4rec_src.inc next to this file's build and compiles this file; the
// kernels then run over block-record chunks made by the oracle, and their
// LZ4 blocks are decoded by the restated reference decoder. Test
// infrastructure only; the product never calls it.
#include "warp_emu.h"

struct LzRegion {
    int a, first_st, first_hdr, last_end, rbytes, ridx, pad0, pad1;
};
namespace cz {
constexpr int kMaskBytes = 4096;
inline unsigned lanemask_lt() { return (1u << emu_lane()) - 1u; }
}  // namespace cz

#define CZ_LZ4REC_NO_LAUNCHERS
#include "lz4rec_src.inc"

#include <vector>

using namespace cz;

extern "C" int emu_lz4rec_smem_bytes(void) { return (int)sizeof(lzr::Smem) * lzr::kWarps; }

// The whole LZ4 stage of nchunks chunks: regions (ctas CTAs of kWarps warps,
// grid-stride as on the GPU), sizes, stitch into out at dst_off (filled here
// from the sizes). Returns 0, or -1 when a chunk size is negative.
extern "C" int emu_lz4rec(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                          const int *rec_bytes, const long long *blk_dst, long long nblocks, int bpc, int shuffle,
                          uint8_t *lz, const long long *lz_off, LzRegion *reg, int *out_len, uint8_t *out,
                          long long *dst_off, int ctas, unsigned seed)
{
    std::vector<unsigned char> smem(sizeof(lzr::Smem) * lzr::kWarps);
    g_emu_smem = smem.data();
    gridDim.x = (unsigned)ctas;
    blockDim.x = lzr::kWarps * 32;
    for (int b = 0; b < ctas; ++b)
        for (int wib = 0; wib < lzr::kWarps; ++wib) {
            blockIdx.x = (unsigned)b;
            emu_run_warp((unsigned)wib * 32, seed + (unsigned)(b * lzr::kWarps + wib), [&] {
                lzr::lz4_region_kernel(in, in_off, in_len, nchunks, rec_bytes, blk_dst, nblocks, bpc, shuffle, lz,
                                       lz_off, reg);
            });
        }
    blockIdx.x = 0;
    blockDim.x = 1u << 30;
    for (int c = 0; c < nchunks; ++c) {
        threadIdx.x = (unsigned)c;
        lzr::lz4_region_sizes(reg, in_len, nchunks, 3 * bpc, out_len);
    }
    dst_off[0] = 0;
    for (int c = 0; c < nchunks; ++c) {
        if (out_len[c] < 0) return -1;
        dst_off[c + 1] = dst_off[c] + out_len[c];
    }
    blockDim.x = 32;
    gridDim.x = (unsigned)nchunks;
    for (int c = 0; c < nchunks; ++c) {
        blockIdx.x = (unsigned)c;
        emu_run_warp(0, seed, [&] { lzr::lz4_stitch_kernel(in, in_off, in_len, nchunks, 3 * bpc, lz, lz_off, reg, out, dst_off); });
    }
    return 0;
}
