// cz_stream.cu -- device-side stream assembly: chunk layout, record packing,
// offset scans and record location in decoded chunks.
//
// The writer groups consecutive block records [int32 nbytes][record] into
// chunks that are compressed independently and placed back to back; a LUT of
// chunk offsets follows (SerializerIO_WaveletCompression_MPI_Simple.h:101-184,
// 236-240, 574-591). Here chunk offsets come from a device prefix sum instead
// of the reference's omp-critical offset allocation and MPI_Exscan (:138-159,
// :389). The reader finds a block by walking the nbytes headers of its
// decoded chunk up to its subid (Reader_WaveletCompression.h:665-673).
#include "cz_codec.h"
#include "cz_device.cuh"

namespace cz {

__global__ void chunk_setup_kernel(int bpc, long long nblocks, int nchunks, const int *rec_bytes, long long *in_off,
                                   int *in_len, long long *blk_dst, long long *lz_off, long long lz_slot)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long g0 = (long long)c * bpc;
    const long long base = bpc == 1 ? g0 * kSlotBytes : (long long)c * bpc * kSlotBytes;
    long long acc = 0;
    for (long long g = g0; g < g0 + bpc && g < nblocks; ++g) {
        if (blk_dst) blk_dst[g] = base + acc;
        acc += 4 + rec_bytes[g];
    }
    in_off[c] = base;
    in_len[c] = (int)acc;
    lz_off[c] = (long long)c * lz_slot;
}

// One CTA per block: copy [nbytes][record] with 16-byte moves when aligned.
__global__ void pack_records_kernel(const uint8_t *__restrict__ stage, const int *rec_bytes,
                                    const long long *blk_dst, uint8_t *__restrict__ chunk_in)
{
    const long long g = blockIdx.x;
    const int n = 4 + rec_bytes[g];
    const uint8_t *s = stage + g * (long long)kSlotBytes;
    uint8_t *d = chunk_in + blk_dst[g];
    if ((reinterpret_cast<uintptr_t>(d) & 15) == 0) {
        const int n16 = n >> 4;
        for (int i = threadIdx.x; i < n16; i += blockDim.x)
            reinterpret_cast<uint4 *>(d)[i] = reinterpret_cast<const uint4 *>(s)[i];
        for (int i = (n16 << 4) + threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    } else {
        // records are multiples of 4 bytes, so 4-byte moves always line up
        const int n4 = n >> 2;
        for (int i = threadIdx.x; i < n4; i += blockDim.x)
            reinterpret_cast<uint32_t *>(d)[i] = reinterpret_cast<const uint32_t *>(s)[i];
    }
}

// Single-CTA exclusive scan (chunk counts are at most a few hundred thousand).
__global__ void __launch_bounds__(1024) scan_kernel(const int *len, int n, long long *off, int carry_in)
{
    __shared__ long long warp_sum[32];
    __shared__ long long carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = carry_in ? off[0] : 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const long long v = i < n ? (long long)len[i] : 0;
        long long incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            long long w = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            warp_sum[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const long long before = carry + (warp ? warp_sum[warp - 1] : 0);
        if (i < n) off[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[n] = carry;
}

// One thread per chunk walks its records (lz4.c output or raw chunk).
__global__ void locate_records_kernel(int bpc, long long nblocks, int nchunks, const long long *chunk_base,
                                      const int *dec_len, long long *rec_off, int *status, const uint8_t *base)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long g0 = (long long)c * bpc;
    const long long cb = chunk_base[c];
    const int len = dec_len[c];
    long long pos = 0;
    bool ok = len >= 0;
    for (long long g = g0; g < g0 + bpc && g < nblocks; ++g) {
        int nb = -1;
        if (ok && pos + 4 <= len) nb = *reinterpret_cast<const int *>(base + cb + pos);
        if (!ok || nb < kMaskBytes || nb > kMaxRecord + 4 || pos + 4 + nb > len) {
            ok = false;
            rec_off[g] = -1;
            status[g] = -1;
            continue;
        }
        rec_off[g] = cb + pos;
        status[g] = 0;
        pos += 4 + nb;
    }
}

// Decode-side chunk geometry: input sizes from the offset table, decoded
// chunk c at c*dec_cap (LZ4) or in place (raw).
__global__ void decode_setup_kernel(int nchunks, const long long *off, int *in_len, long long *dec_off, int *dec_cap,
                                    long long cap, int raw)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long n = off[c + 1] - off[c];
    in_len[c] = (n < 0 || n > 0x7fffffffLL) ? -1 : (int)n;
    dec_off[c] = raw ? off[c] : (long long)c * cap;
    dec_cap[c] = (int)cap;
}

// General record location: per chunk, the offsets of its first maxsub
// records; then per block, its record from (chunk, subid).
__global__ void chunk_records_kernel(int nchunks, int maxsub, const long long *chunk_base, const int *dec_len,
                                     const uint8_t *base, long long *chunk_rec)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long cb = chunk_base[c];
    const int len = dec_len[c];
    long long pos = 0;
    bool ok = len >= 0;
    for (int k = 0; k < maxsub; ++k) {
        int nb = -1;
        if (ok && pos + 4 <= len) nb = *reinterpret_cast<const int *>(base + cb + pos);
        if (!ok || nb < kMaskBytes || nb > kMaxRecord + 4 || pos + 4 + nb > len) {
            ok = false;
            chunk_rec[(long long)c * maxsub + k] = -1;
            continue;
        }
        chunk_rec[(long long)c * maxsub + k] = cb + pos;
        pos += 4 + nb;
    }
}

__global__ void map_blocks_kernel(long long nblocks, int nchunks, int maxsub, const int *block_chunk,
                                  const int *block_subid, const long long *chunk_rec, long long *rec_off)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= nblocks) return;
    const int c = block_chunk[g], k = block_subid[g];
    rec_off[g] = (c < 0 || c >= nchunks || k < 0 || k >= maxsub) ? -1 : chunk_rec[(long long)c * maxsub + k];
}

// min over the per-block status words (0 ok, negative error) into *flag.
__global__ void status_reduce_kernel(const int *status, long long n, int *flag)
{
    int worst = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        worst = min(worst, status[i]);
#pragma unroll
    for (int o = 16; o; o >>= 1) worst = min(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    if ((threadIdx.x & 31) == 0 && worst < 0) atomicMin(flag, worst);
}

__global__ void neg_reduce_kernel(const int *v, int n, int *flag)
{
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) bad |= v[i] < 0;
    if (bad) atomicMin(flag, -1);
}

__global__ void rebase_kernel(long long *off, int n, long long base)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) off[i] -= base;
}

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_rebase(long long *off, int n, long long base, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    rebase_kernel<<<(n + 255) / 256, 256, 0, st>>>(off, n, base);
    return cudaGetLastError();
}

cudaError_t cz_launch_decode_setup(int nchunks, const long long *off, int *in_len, long long *dec_off, int *dec_cap,
                                   long long cap, int raw, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    decode_setup_kernel<<<(nchunks + 255) / 256, 256, 0, st>>>(nchunks, off, in_len, dec_off, dec_cap, cap, raw);
    return cudaGetLastError();
}

cudaError_t cz_launch_chunk_records(int nchunks, int maxsub, const long long *chunk_base, const int *dec_len,
                                    const uint8_t *base, long long *chunk_rec, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    chunk_records_kernel<<<(nchunks + 127) / 128, 128, 0, st>>>(nchunks, maxsub, chunk_base, dec_len, base, chunk_rec);
    return cudaGetLastError();
}

cudaError_t cz_launch_map_blocks(long long nblocks, int nchunks, int maxsub, const int *block_chunk,
                                 const int *block_subid, const long long *chunk_rec, long long *rec_off,
                                 cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    map_blocks_kernel<<<(unsigned)((nblocks + 255) / 256), 256, 0, st>>>(nblocks, nchunks, maxsub, block_chunk,
                                                                        block_subid, chunk_rec, rec_off);
    return cudaGetLastError();
}

cudaError_t cz_launch_status_reduce(const int *status, long long n, int *flag, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const long long b = (n + 255) / 256;
    status_reduce_kernel<<<(unsigned)(b < 1024 ? b : 1024), 256, 0, st>>>(status, n, flag);
    return cudaGetLastError();
}

cudaError_t cz_launch_neg_reduce(const int *v, int n, int *flag, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int b = (n + 255) / 256;
    neg_reduce_kernel<<<b < 1024 ? b : 1024, 256, 0, st>>>(v, n, flag);
    return cudaGetLastError();
}

cudaError_t cz_launch_chunk_setup(int bpc, long long nblocks, int nchunks, const int *rec_bytes, long long *in_off,
                                  int *in_len, long long *blk_dst, long long *lz_off, long long lz_slot,
                                  cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    chunk_setup_kernel<<<(nchunks + 255) / 256, 256, 0, st>>>(bpc, nblocks, nchunks, rec_bytes, in_off, in_len,
                                                               blk_dst, lz_off, lz_slot);
    return cudaGetLastError();
}

cudaError_t cz_launch_pack_records(const uint8_t *stage, const int *rec_bytes, long long nblocks,
                                   const long long *blk_dst, uint8_t *chunk_in, cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    pack_records_kernel<<<(unsigned)nblocks, 256, 0, st>>>(stage, rec_bytes, blk_dst, chunk_in);
    return cudaGetLastError();
}

cudaError_t cz_launch_scan(const int *len, int n, long long *off, cudaStream_t st)
{
    scan_kernel<<<1, 1024, 0, st>>>(len, n, off, 0);
    return cudaGetLastError();
}

cudaError_t cz_launch_scan_from(const int *len, int n, long long *off, cudaStream_t st)
{
    scan_kernel<<<1, 1024, 0, st>>>(len, n, off, 1);
    return cudaGetLastError();
}

cudaError_t cz_launch_locate_records(int bpc, long long nblocks, int nchunks, const long long *chunk_base,
                                     const int *dec_len, long long *rec_off, int *status, const uint8_t *base,
                                     cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    locate_records_kernel<<<(nchunks + 127) / 128, 128, 0, st>>>(bpc, nblocks, nchunks, chunk_base, dec_len, rec_off,
                                                                  status, base);
    return cudaGetLastError();
}
