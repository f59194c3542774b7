// cz_lz4.cu -- LZ4 legacy block format on the GPU, one warp per chunk.
//
// Encoder: greedy parse, format-compatible with the reference decoder
// LZ4_uncompress_unknownOutputSize (ThirdParty/lz4/lz4.c:802-905): minimum
// match 4, offsets 1..65535, the last 5 bytes are literals and the last
// match starts at least 12 bytes before the end (lz4.c:177-204). Instead of
// probing one position at a time, a warp hashes 32 consecutive positions at
// once (4 KiB-entry table per warp in shared memory), also matches lanes
// against earlier lanes of the same window (__match_any_sync), takes the
// first valid candidate, extends it backwards and forwards 32 bytes per step
// and emits the sequence with a warp-wide copy.
//
// Decoder: the same acceptance tests and error convention as
// LZ4_uncompress_unknownOutputSize (-(input position) on malformed input; an
// empty input yields 0), with warp-wide literal and match copies. Matches
// overlapping their source are copied as the periodic pattern they encode.
#include "cz_codec.h"

namespace cz {

constexpr int kLzWarps = 4;
constexpr int kHashLog = 12;
constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kMinMatch = 4, kLastLiterals = 5, kMfLimit = 12;

__device__ __forceinline__ uint32_t rd32(const uint8_t *p)
{
    // unaligned little-endian 32-bit read via the two covering words
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    const uint32_t lo = __ldg(w);
    if (sh == 0) return lo;
    return __funnelshift_r(lo, __ldg(w + 1), sh);
}

__device__ __forceinline__ uint32_t lz_hash(uint32_t v) { return (v * 2654435761u) >> (32 - kHashLog); }

__device__ __forceinline__ unsigned lanemask_lt_()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Length field continuation bytes: n/255 bytes of 255 then n%255.
__device__ __forceinline__ void put_len(uint8_t *dst, int op, int n, int lane)
{
    const int cnt = n / 255 + 1;
    for (int i = lane; i < cnt; i += 32) dst[op + i] = (uint8_t)(i < cnt - 1 ? 255 : n % 255);
}

__global__ void __launch_bounds__(kLzWarps * 32)
lz4_encode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, int *out_len)
{
    __shared__ uint32_t table_all[kLzWarps][1 << kHashLog];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t *table = table_all[wib];
    const int gw = blockIdx.x * kLzWarps + wib, nw = gridDim.x * kLzWarps;

    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int L = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int cap = L + L / 255 + 16;
        for (int i = lane; i < (1 << kHashLog); i += 32) table[i] = kEmpty;
        __syncwarp();
        int ip = 0, anchor = 0, op = 0;
        bool overflow = false;
        if (L >= kMfLimit + 1) {
            const int mflimit = L - kMfLimit, matchlimit = L - kLastLiterals;
            while (ip <= mflimit) {
                const int p = ip + lane;
                const bool valid = p <= mflimit;
                const uint32_t seq = valid ? rd32(src + p) : 0u;
                const uint32_t h = lz_hash(seq);
                uint32_t cand = valid ? table[h] : kEmpty;
                const unsigned vmask = __ballot_sync(0xffffffffu, valid);
                const unsigned peers = __match_any_sync(0xffffffffu, seq) & lanemask_lt_() & vmask;
                __syncwarp();
                if (valid) table[h] = (uint32_t)p;
                __syncwarp();
                if (peers) cand = (uint32_t)(ip + 31 - __clz(peers));
                const bool ok = valid && cand != kEmpty && (int)cand < p && p - (int)cand <= 65535 &&
                                rd32(src + cand) == seq;
                const unsigned ball = __ballot_sync(0xffffffffu, ok);
                if (!ball) {
                    ip += 32;
                    continue;
                }
                const int f = __ffs(ball) - 1;
                int m = ip + f;
                int ref = __shfl_sync(0xffffffffu, (int)cand, f);
                // catch up backwards over equal bytes (lz4.c:406)
                for (;;) {
                    const int k = lane + 1;
                    const bool eq = (m - k >= anchor) && (ref - k >= 0) && src[m - k] == src[ref - k];
                    const unsigned neq = __ballot_sync(0xffffffffu, !eq);
                    const int back = neq ? __ffs(neq) - 1 : 32;
                    m -= back;
                    ref -= back;
                    if (back < 32) break;
                }
                // extend forwards up to the last-literals limit
                int len = kMinMatch;
                for (;;) {
                    const int q = m + len + lane;
                    const bool eq = q < matchlimit && src[q] == src[ref + len + lane];
                    const unsigned neq = __ballot_sync(0xffffffffu, !eq);
                    const int fw = neq ? __ffs(neq) - 1 : 32;
                    len += fw;
                    if (fw < 32) break;
                }
                const int lit = m - anchor;
                const int need = 1 + (lit >= 15 ? lit / 255 + 1 : 0) + lit + 2 + (len - 4 >= 15 ? (len - 19) / 255 + 1 : 0);
                if (op + need + 1 + kLastLiterals > cap) {
                    overflow = true;
                    break;
                }
                const int ml = len - kMinMatch;
                if (lane == 0) dst[op] = (uint8_t)(((lit >= 15 ? 15 : lit) << 4) | (ml >= 15 ? 15 : ml));
                op += 1;
                if (lit >= 15) {
                    put_len(dst, op, lit - 15, lane);
                    op += (lit - 15) / 255 + 1;
                }
                for (int i = lane; i < lit; i += 32) dst[op + i] = src[anchor + i];
                op += lit;
                const int off = m - ref;
                if (lane == 0) {
                    dst[op] = (uint8_t)off;
                    dst[op + 1] = (uint8_t)(off >> 8);
                }
                op += 2;
                if (ml >= 15) {
                    put_len(dst, op, ml - 15, lane);
                    op += (ml - 15) / 255 + 1;
                }
                ip = m + len;
                anchor = ip;
                // the reference seeds the table with ip-2 after a match (lz4.c:458)
                if (ip <= mflimit && lane == 0) table[lz_hash(rd32(src + ip - 2))] = (uint32_t)(ip - 2);
                __syncwarp();
            }
        }
        if (!overflow) {
            const int lit = L - anchor;
            const int need = 1 + (lit >= 15 ? lit / 255 + 1 : 0) + lit;
            if (op + need > cap) {
                overflow = true;
            } else {
                if (lane == 0) dst[op] = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
                op += 1;
                if (lit >= 15) {
                    put_len(dst, op, lit - 15, lane);
                    op += (lit - 15) / 255 + 1;
                }
                for (int i = lane; i < lit; i += 32) dst[op + i] = src[anchor + i];
                op += lit;
            }
        }
        if (lane == 0) out_len[c] = overflow ? -1 : op;
        __syncwarp();
    }
}

// Reads a run of length-continuation bytes starting at ip (while bytes are
// 255 and ip < lim); returns the sum and advances ip past the last byte read.
// stop_after_non255: the run ends with the first byte that is not 255.
__device__ __forceinline__ long long get_len(const uint8_t *src, int &ip, int lim, int lane)
{
    long long sum = 0;
    for (;;) {
        const int q = ip + lane;
        const int b = q < lim ? (int)src[q] : -1;
        const unsigned stop = __ballot_sync(0xffffffffu, b != 255);
        const int n = stop ? __ffs(stop) - 1 : 32;  // 255-bytes before the stop
        sum += 255LL * n;
        if (!stop) {
            ip += 32;
            continue;
        }
        const int bs = __shfl_sync(0xffffffffu, b, n);
        if (bs < 0) {  // ran into the limit: all bytes before it were read
            ip += n;
            return sum;
        }
        sum += bs;
        ip += n + 1;
        return sum;
    }
}

__global__ void __launch_bounds__(128)
lz4_decode_kernel(const uint8_t *__restrict__ in, const long long *in_off, const int *in_len, int nchunks,
                  uint8_t *__restrict__ out, const long long *out_off, const int *out_cap, int *out_len)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = gw; c < nchunks; c += nw) {
        const uint8_t *src = in + in_off[c];
        const int iend = in_len[c];
        uint8_t *dst = out + out_off[c];
        const int oend = out_cap[c];
        int ip = 0, op = 0, err = 0;
        if (iend <= 0) {
            if (lane == 0) out_len[c] = 0;  // lz4.c:836: error exit at position 0
            continue;
        }
        for (;;) {
            const int token = src[ip++];
            long long len = token >> 4;
            if (len == 15) len += get_len(src, ip, iend, lane);
            // lz4.c:851-858: the last sequence is literals only and ends the input
            if (len > (long long)(oend - op - kMfLimit) || len > (long long)(iend - ip - (2 + 1 + kLastLiterals))) {
                if (len > (long long)(oend - op) || len != (long long)(iend - ip)) {
                    err = 1;
                    break;
                }
                for (int i = lane; i < (int)len; i += 32) dst[op + i] = src[ip + i];
                op += (int)len;
                break;
            }
            for (int i = lane; i < (int)len; i += 32) dst[op + i] = src[ip + i];
            op += (int)len;
            ip += (int)len;
            const int off = (int)src[ip] | ((int)src[ip + 1] << 8);
            ip += 2;
            if (off == 0 || off > op) {
                err = 1;
                break;
            }
            long long ml = token & 15;
            if (ml == 15) {
                // lz4.c:873-882: continuation bytes only while ip < iend-(LASTLITERALS+1)
                int q = ip;
                long long add = 0;
                const int lim = iend - (kLastLiterals + 1);
                for (;;) {
                    const int pos = q + lane;
                    const int b = pos < lim ? (int)src[pos] : -1;
                    const unsigned stop = __ballot_sync(0xffffffffu, b != 255);
                    const int n = stop ? __ffs(stop) - 1 : 32;
                    add += 255LL * n;
                    if (!stop) {
                        q += 32;
                        continue;
                    }
                    const int bs = __shfl_sync(0xffffffffu, b, n);
                    if (bs >= 0) {
                        add += bs;
                        q += n + 1;
                    } else {
                        q += n;
                    }
                    break;
                }
                ip = q;
                ml += add;
            }
            ml += kMinMatch;
            if (ml > (long long)(oend - op - kLastLiterals)) {  // lz4.c:888-890
                err = 1;
                break;
            }
            __syncwarp();
            for (int i = lane; i < (int)ml; i += 32) dst[op + i] = __ldcg(dst + op - off + (i % off));
            op += (int)ml;
            __syncwarp();
        }
        if (lane == 0) out_len[c] = err ? -(ip > 0 ? ip : 1) : op;
        __syncwarp();
    }
}

__global__ void gather_kernel(const uint8_t *__restrict__ src, const long long *src_off, const int *len,
                              uint8_t *__restrict__ dst, const long long *dst_off)
{
    const int c = blockIdx.x;
    const int n = len[c];
    const uint8_t *s = src + src_off[c];
    uint8_t *d = dst + dst_off[c];
    for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
}

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_lz4_encode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, int *out_len, int grid, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    lz4_encode_kernel<<<grid, kLzWarps * 32, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_len);
    return cudaGetLastError();
}

cudaError_t cz_launch_lz4_decode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, const int *out_cap, int *out_len, int grid,
                                 cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    lz4_decode_kernel<<<grid, 128, 0, st>>>(in, in_off, in_len, nchunks, out, out_off, out_cap, out_len);
    return cudaGetLastError();
}

cudaError_t cz_launch_gather(const uint8_t *src, const long long *src_off, const int *len, int nchunks,
                             uint8_t *dst, const long long *dst_off, cudaStream_t st)
{
    if (nchunks <= 0) return cudaSuccess;
    gather_kernel<<<nchunks, 256, 0, st>>>(src, src_off, len, dst, dst_off);
    return cudaGetLastError();
}
