// cz_codec.cu -- the block codec kernels.
//
// encode: field blocks -> [int32 nbytes][4096-byte mask][survivors] records,
//   fusing the reference's WaveletCompressor::compress sequence
//   (WaveletCompressor.cpp:152-182): fwt (FullWaveletTransform.h:44-49),
//   threshold with the coarse-first survivor order (:58-96),
//   serialize_bitset (WaveletCompressor.cpp:96-122), float_zero_bits3
//   (:33-43) and shuffle3 (:55-73), plus the record framing of the writer's
//   block loop (SerializerIO_WaveletCompression_MPI_Simple.h:236-240).
// decode: records -> field blocks, the reference's decompress
//   (WaveletCompressor.cpp:231-259): deserialize_bitset, reshuffle3, load
//   (FullWaveletTransform.h:99-150) and iwt.
//
// One CTA per SM, persistent; blocks are taken from a device work queue so
// one launch serves one field or a batch of uneven fields. A block is held
// whole in shared memory (128 KiB, swizzled); while a block is thresholded
// and emitted, the next block's 128 KiB is already in flight into registers.
#include "cz_codec.h"
#include "cz_device.cuh"

namespace cz {

#ifndef CZ_CODEC_THREADS
#define CZ_CODEC_THREADS 256
#endif
constexpr int kNT = CZ_CODEC_THREADS;  // threads per CTA (one CTA per SM)
constexpr int kNW = kNT / 32;
constexpr int kChunksPerWarp = 1024 / kNW;  // 32-entry survivor-order chunks
constexpr int kPrefetch = (kBS3 / 4) / kNT;  // float4 per thread per block

// shared memory map (bytes)
constexpr int kSmBlock = 0;
constexpr int kSmMask = kBS3 * 4;
constexpr int kSmBallot = kSmMask + kMaskBytes;
constexpr int kSmWarp = kSmBallot + 1024 * 4;
constexpr int kSmBytes = kSmWarp + 64 * 4;

struct BlockRef {
    const CzField *f;
    int bx, by, bz;
};

__device__ __forceinline__ BlockRef locate(const CzField *fields, int nfields, long long g)
{
    int lo = 0, hi = nfields - 1;
    while (lo < hi) {  // last field with block0 <= g
        const int mid = (lo + hi + 1) >> 1;
        if (fields[mid].block0 <= g) lo = mid;
        else hi = mid - 1;
    }
    const CzField *f = &fields[lo];
    const long long b = g - f->block0;
    const int nbx = f->nx >> 5, nby = f->ny >> 5;
    BlockRef r;
    r.f = f;
    r.bx = (int)(b % nbx);
    r.by = (int)((b / nbx) % nby);
    r.bz = (int)(b / ((long long)nbx * nby));
    return r;
}

__device__ __forceinline__ const float *row_ptr(const BlockRef &r, int y, int z)
{
    const CzField &f = *r.f;
    return f.data + ((size_t)(r.bz * 32 + z) * f.ny + (size_t)(r.by * 32 + y)) * f.nx + r.bx * 32;
}

__device__ __forceinline__ void prefetch_block(const BlockRef &r, float4 (&pf)[kPrefetch])
{
#pragma unroll
    for (int k = 0; k < kPrefetch; ++k) {
        const int i = threadIdx.x + k * kNT;
        const int row = i >> 3, c = i & 7;
        pf[k] = __ldcs(reinterpret_cast<const float4 *>(row_ptr(r, row & 31, row >> 5)) + c);
    }
}

__device__ __forceinline__ void stage_block(float *sb, const float4 (&pf)[kPrefetch])
{
#pragma unroll
    for (int k = 0; k < kPrefetch; ++k) {
        const int i = threadIdx.x + k * kNT;
        const int row = i >> 3, x0 = (i & 7) * 4;
        const int y = row & 31, z = row >> 5;
        sb[swz(x0 + 0, y, z)] = pf[k].x;
        sb[swz(x0 + 1, y, z)] = pf[k].y;
        sb[swz(x0 + 2, y, z)] = pf[k].z;
        sb[swz(x0 + 3, y, z)] = pf[k].w;
    }
}

// Block-wide exclusive scan of one count per warp; returns the warp's offset
// and the total through *total.
__device__ __forceinline__ int warp_offsets(int *swarp, int cnt, int *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) swarp[warp] = cnt;
    __syncthreads();
    if (warp == 0) {
        int v = lane < kNW ? swarp[lane] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane < kNW) swarp[32 + lane] = incl - v;
        if (lane == kNW - 1) swarp[32 + kNW] = incl;
    }
    __syncthreads();
    *total = swarp[32 + kNW];
    return swarp[32 + warp];
}

template <int KIND>
__global__ void __launch_bounds__(kNT, 1)
encode_kernel(const CzField *fields, int nfields, long long total_blocks, int zerobits, int shuffle,
              uint8_t *stage, int *rec_bytes, unsigned long long *queue)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *sb = reinterpret_cast<float *>(smem + kSmBlock);
    uint8_t *smask = smem + kSmMask;
    unsigned *sballot = reinterpret_cast<unsigned *>(smem + kSmBallot);
    int *swarp = reinterpret_cast<int *>(smem + kSmWarp);
    __shared__ long long s_ticket;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t zmask = zerobits > 0 ? ~((1u << zerobits) - 1u) : 0xffffffffu;

    if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(queue, 1ull);
    __syncthreads();
    long long g = s_ticket;
    float4 pf[kPrefetch];
    if (g < total_blocks) prefetch_block(locate(fields, nfields, g), pf);

    while (g < total_blocks) {
        const BlockRef ref = locate(fields, nfields, g);
        const float eps = ref.f->eps;
        __syncthreads();  // the previous block's emit is done with smem
        stage_block(sb, pf);
        __syncthreads();
        forward_transform<KIND, kNT>(sb);

        // next ticket; its loads overlap thresholding and emission
        if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        const long long gn = s_ticket;
        if (gn < total_blocks) prefetch_block(locate(fields, nfields, gn), pf);

        // ---- pass 1: keep flags in survivor order, mask bytes, counts
        int cnt = 0;
        for (int ch = 0; ch < kChunksPerWarp; ++ch) {
            const int cidx = warp * kChunksPerWarp + ch;
            const int s = cidx * 32 + lane;
            int p;
            const float v = sb[swz_of_stream(s, p)];
            const bool keep = s < 64 || fabsf(v) > eps;  // FullWaveletTransform.h:84
            const unsigned b = __ballot_sync(0xffffffffu, keep);
            if (lane == 0) sballot[cidx] = b;
            cnt += __popc(b);
            // mask bit p is LSB-first in byte p>>3 (WaveletCompressor.cpp:103-111);
            // level-32 runs are 16 positions along px, level-16 runs 8
            if (s >= 4096) {
                if ((lane & 15) == 0) reinterpret_cast<uint16_t *>(smask)[p >> 4] = (uint16_t)(b >> lane);
            } else if (s >= 512) {
                if ((lane & 7) == 0) smask[p >> 3] = (uint8_t)(b >> lane);
            }
        }
        // coarse and level-8 positions: the 64 mask bytes with px,py,pz < 8
        if (threadIdx.x < 64) {
            const int py = threadIdx.x & 7, pz = threadIdx.x >> 3;
            unsigned byte = 0;
#pragma unroll
            for (int px = 0; px < 8; ++px) {
                const bool coarse = px < 4 && py < 4 && pz < 4;
                byte |= (unsigned)(coarse || fabsf(sb[swz(px, py, pz)]) > eps) << px;
            }
            smask[(py + 32 * pz) * 4] = (uint8_t)byte;
        }
        int S;
        int base = warp_offsets(swarp, cnt, &S);
        const int nb = kMaskBytes + 4 * S;
        uint8_t *slot = stage + (size_t)g * kSlotBytes;
        if (threadIdx.x == 0) {
            *reinterpret_cast<int *>(slot) = nb;
            rec_bytes[g] = nb;
        }
        {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(smask);
            uint32_t *dst = reinterpret_cast<uint32_t *>(slot + 4);
            for (int i = threadIdx.x; i < kMaskBytes / 4; i += kNT) dst[i] = src[i];
        }
        // ---- pass 2: survivors in order, zero-bits, optional byte planes
        uint8_t *pay = slot + 4 + kMaskBytes;
        for (int ch = 0; ch < kChunksPerWarp; ++ch) {
            const int cidx = warp * kChunksPerWarp + ch;
            const unsigned b = sballot[cidx];
            if ((b >> lane) & 1u) {
                const int s = cidx * 32 + lane;
                int p;
                const uint32_t u = __float_as_uint(sb[swz_of_stream(s, p)]) & zmask;
                const int k = base + __popc(b & lanemask_lt());
                if (shuffle) {
                    pay[k] = (uint8_t)u;
                    pay[S + k] = (uint8_t)(u >> 8);
                    pay[2 * S + k] = (uint8_t)(u >> 16);
                    pay[3 * S + k] = (uint8_t)(u >> 24);
                } else {
                    reinterpret_cast<uint32_t *>(pay)[k] = u;
                }
            }
            base += __popc(b);
        }
        g = gn;
    }
}

template <int KIND>
__global__ void __launch_bounds__(kNT, 1)
decode_kernel(const CzField *fields, int nfields, long long total_blocks, int shuffle, const uint8_t *base,
              const long long *rec_off, int *status, unsigned long long *queue)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *sb = reinterpret_cast<float *>(smem + kSmBlock);
    uint8_t *smask = smem + kSmMask;
    unsigned *sballot = reinterpret_cast<unsigned *>(smem + kSmBallot);
    int *swarp = reinterpret_cast<int *>(smem + kSmWarp);
    __shared__ long long s_ticket;
    __shared__ int s_bad;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            s_ticket = (long long)atomicAdd(queue, 1ull);
            s_bad = 0;
        }
        __syncthreads();
        const long long g = s_ticket;
        if (g >= total_blocks) break;
        const BlockRef ref = locate(fields, nfields, g);
        const long long ro = rec_off[g];
        const uint8_t *slot = base + (ro < 0 ? 0 : ro);
        const int nb = ro < 0 ? -1 : *reinterpret_cast<const int *>(slot);
        const bool size_ok = nb >= kMaskBytes && nb <= kMaxRecord + 4;

        // deserialize_bitset (WaveletCompressor.cpp:124-150) + popcount
        int ones = 0;
        {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(slot + 4);
            uint32_t *dst = reinterpret_cast<uint32_t *>(smask);
            for (int i = threadIdx.x; i < kMaskBytes / 4; i += kNT) {
                const uint32_t w = size_ok ? src[i] : 0u;
                dst[i] = w;
                ones += __popc(w);
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) ones += __shfl_xor_sync(0xffffffffu, ones, o);
        int expected;
        warp_offsets(swarp, ones, &expected);
        const int payload = nb - kMaskBytes;
        int nel = payload / 4;
        if (nel - expected == 1) nel--;  // :247-250
        // every coarse bit set (the base case reads 64 survivors, :178-189)
        if (threadIdx.x < 64) {
            const int x = threadIdx.x & 3, y = (threadIdx.x >> 2) & 3, z = threadIdx.x >> 4;
            const int p = x + 32 * (y + 32 * z);
            if (!((smask[p >> 3] >> (p & 7)) & 1)) s_bad = 1;
        }
        __syncthreads();
        const bool ok = size_ok && nel == expected && !s_bad;
        if (threadIdx.x == 0) status[g] = ok ? 0 : -1;

        // pass 1: survivor ranks in the coarse-first order
        int cnt = 0;
        for (int ch = 0; ch < kChunksPerWarp; ++ch) {
            const int cidx = warp * kChunksPerWarp + ch;
            const int s = cidx * 32 + lane;
            int px, py, pz;
            pos_of_stream(s, px, py, pz);
            const int p = px + 32 * (py + 32 * pz);
            const bool eat = ok && ((smask[p >> 3] >> (p & 7)) & 1);
            const unsigned b = __ballot_sync(0xffffffffu, eat);
            if (lane == 0) sballot[cidx] = b;
            cnt += __popc(b);
        }
        int total;
        int base = warp_offsets(swarp, cnt, &total);
        // pass 2: FullTransformEngine::load -- survivors to their positions,
        // zeros elsewhere; reshuffle3 (:75-93) reads byte planes of c = n/4
        const uint8_t *pay = slot + 4 + kMaskBytes;
        const int c = payload / 4;
        for (int ch = 0; ch < kChunksPerWarp; ++ch) {
            const int cidx = warp * kChunksPerWarp + ch;
            const unsigned b = sballot[cidx];
            const int s = cidx * 32 + lane;
            int p;
            const int a = swz_of_stream(s, p);
            float v = 0.f;
            if ((b >> lane) & 1u) {
                const int k = base + __popc(b & lanemask_lt());
                uint32_t u;
                if (shuffle)
                    u = (uint32_t)pay[k] | ((uint32_t)pay[c + k] << 8) | ((uint32_t)pay[2 * c + k] << 16) |
                        ((uint32_t)pay[3 * c + k] << 24);
                else
                    u = reinterpret_cast<const uint32_t *>(pay)[k];
                v = __uint_as_float(u);
            }
            sb[a] = v;
            base += __popc(b);
        }
        __syncthreads();
        inverse_transform<KIND, kNT>(sb);
        // copy_to (WaveletCompressor.h:73-82) into the field, x fastest
        float *out = const_cast<float *>(ref.f->data);
        const CzField &f = *ref.f;
        for (int i = threadIdx.x; i < kBS3 / 4; i += kNT) {
            const int row = i >> 3, x0 = (i & 7) * 4;
            const int y = row & 31, z = row >> 5;
            float4 w;
            w.x = sb[swz(x0 + 0, y, z)];
            w.y = sb[swz(x0 + 1, y, z)];
            w.z = sb[swz(x0 + 2, y, z)];
            w.w = sb[swz(x0 + 3, y, z)];
            float *dst = out + ((size_t)(ref.bz * 32 + z) * f.ny + (size_t)(ref.by * 32 + y)) * f.nx + ref.bx * 32 + x0;
            __stcs(reinterpret_cast<float4 *>(dst), w);
        }
    }
}

}  // namespace cz

using namespace cz;

extern "C" int cz_codec_smem_bytes(void) { return kSmBytes; }

template <int KIND>
static cudaError_t launch_encode(const CzField *fields, int nfields, long long total_blocks, int zerobits,
                                 int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue, int grid,
                                 cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(encode_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    encode_kernel<KIND><<<grid, kNT, kSmBytes, st>>>(fields, nfields, total_blocks, zerobits, shuffle, stage,
                                                     rec_bytes, queue);
    return cudaGetLastError();
}

template <int KIND>
static cudaError_t launch_decode(const CzField *fields, int nfields, long long total_blocks, int shuffle,
                                 const uint8_t *base, const long long *rec_off, int *status,
                                 unsigned long long *queue, int grid, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(decode_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    decode_kernel<KIND><<<grid, kNT, kSmBytes, st>>>(fields, nfields, total_blocks, shuffle, base, rec_off, status,
                                                     queue);
    return cudaGetLastError();
}

cudaError_t cz_launch_encode(int wtype, const CzField *fields, int nfields, long long total_blocks, int zerobits,
                             int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue, int grid,
                             cudaStream_t st)
{
    switch (wkind(wtype)) {
    case 1: return launch_encode<1>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st);
    case 2: return launch_encode<2>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st);
    default: return launch_encode<3>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st);
    }
}

cudaError_t cz_launch_decode(int wtype, const CzField *fields, int nfields, long long total_blocks, int shuffle,
                             const uint8_t *base, const long long *rec_off, int *status, unsigned long long *queue,
                             int grid, cudaStream_t st)
{
    switch (wkind(wtype)) {
    case 1: return launch_decode<1>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st);
    case 2: return launch_decode<2>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st);
    default: return launch_decode<3>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st);
    }
}
