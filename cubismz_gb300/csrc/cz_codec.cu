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
// One CTA of 512 threads per SM, persistent; blocks come from a device work
// queue, so one launch serves one field or a batch of uneven fields.
//
// Block layout in shared memory: coefficient (x,y,z) at x + 33y + 1057z. Lines
// along any axis are read with immediate offsets and hit 32 distinct banks
// (lane strides 33 and 1057 are 1 mod 32).
//
// Thresholding is fused into the last sweep of each level: the thread that
// finishes a line holds exactly one run of the reference's survivor order
// per octant (16 coefficients along z at level 32, 8 along y at level 16, 4
// along x at level 8, cz_layout.cuh) and the matching bits of one mask word,
// so it records a keep mask per run and its mask bits. One scan over the run
// counts gives every run's output offset; one pass then writes the survivors.
//
// Encode pipeline per block: the x sweep takes its lines from registers that
// were loaded while the previous block was finishing (levels 16/8, scan and
// emission), so HBM reads overlap compute.
#include "cz_block.cuh"

namespace cz {

// SPLIT: the next block's rows are loaded by the warps level 16 leaves idle
// during level 16 and by the others after it; otherwise every thread loads
// its rows after level 32 (one of the autotuner's shapes).
template <int KIND, bool SPLIT>
__device__ __forceinline__ void encode_body(const CzField *fields, int nfields, long long total_blocks, int zerobits,
                                            int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Shared s = carve(smem);
    __shared__ long long s_ticket;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t zmask = zerobits > 0 ? ~((1u << zerobits) - 1u) : 0xffffffffu;

    if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(queue, 1ull);
    __syncthreads();
    long long g = s_ticket;
    float4 pf[16];
    if (g < total_blocks) load_rows(locate(fields, nfields, g), pf);

    while (g < total_blocks) {
        const BlockRef ref = locate(fields, nfields, g);
        const float eps = ref.f->eps;
        __syncthreads();  // the previous block's emission is done with smem
        if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(queue, 1ull);
        // ---- level 32, x lines straight from the prefetched rows
        {
            const int y = threadIdx.x & 31, z = threadIdx.x >> 5;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                float v[32];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    v[4 * k + 0] = pf[8 * r + k].x;
                    v[4 * k + 1] = pf[8 * r + k].y;
                    v[4 * k + 2] = pf[8 * r + k].z;
                    v[4 * k + 3] = pf[8 * r + k].w;
                }
                line_fwd<32, KIND>(v);
                st_line<32, 0>(s.sb, pidx(0, y, z + 16 * r), v);
            }
        }
        __syncthreads();
        const long long gn = s_ticket;
        sweep<32, 1, true, KIND>(s.sb);
        __syncthreads();
        // ---- level 32, z lines + run masks
        for (int l = threadIdx.x; l < 1024; l += kNT) {
            const int x = l & 31, y = l >> 5;
            const int base = pidx(x, y, 0);
            float v[32];
            ld_line<32, 2>(s.sb, base, v);
            line_fwd<32, KIND>(v);
            st_line<32, 2>(s.sb, base, v);
            emit32(s, x, y, keep_bits<32>(v, eps));
        }
        __syncthreads();
        // the next block's rows load while this one finishes: the warps
        // that level 16 leaves idle (threads >= 256) now, the others once
        // level 16 is done
        if ((!SPLIT || threadIdx.x >= 256) && gn < total_blocks) load_rows(locate(fields, nfields, gn), pf);
        // ---- level 16 (z, x, y) on the [0,16)^3 corner
        sweep<16, 2, true, KIND>(s.sb);
        __syncthreads();
        sweep<16, 0, true, KIND>(s.sb);
        __syncthreads();
        if (threadIdx.x < 256) {
            const int x = threadIdx.x & 15, z = threadIdx.x >> 4;
            const int base = pidx(x, 0, z);
            float v[16];
            ld_line<16, 1>(s.sb, base, v);
            line_fwd<16, KIND>(v);
            st_line<16, 1>(s.sb, base, v);
            emit16(s, x, z, keep_bits<16>(v, eps));
        }
        __syncthreads();
        if (SPLIT && threadIdx.x < 256 && gn < total_blocks) load_rows(locate(fields, nfields, gn), pf);
        // ---- level 8 (y, z, x) on the [0,8)^3 corner
        sweep<8, 1, true, KIND>(s.sb);
        __syncthreads();
        sweep<8, 2, true, KIND>(s.sb);
        __syncthreads();
        if (threadIdx.x < 64) {
            const int y = threadIdx.x & 7, z = threadIdx.x >> 3;
            const int base = pidx(0, y, z);
            float v[8];
            ld_line<8, 0>(s.sb, base, v);
            line_fwd<8, KIND>(v);
            st_line<8, 0>(s.sb, base, v);
            emit8(s, y, z, keep_bits<8>(v, eps));
        }
        __syncthreads();
        emit_record(s, g, zmask, shuffle, stage, rec_bytes);
        g = gn;
    }
}

// One CTA per SM with the whole register file.
template <int KIND, bool SPLIT>
__global__ void __launch_bounds__(kNT, 1)
encode_kernel(const CzField *fields, int nfields, long long total_blocks, int zerobits, int shuffle,
              uint8_t *stage, int *rec_bytes, unsigned long long *queue)
{
    encode_body<KIND, SPLIT>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue);
}

// Error statistics of a decoded block against a reference field (the
// quantities of cz2diff, Tools/cz2diff.cpp:116-261): per block
// {e_inf, n_inf, e_1, n_1, e_2, n_2, min, max} with e = |decoded - ref|,
// n = |ref|. The difference is exact (two-sum), maxima are exact, the sums
// are compensated binary32 per thread and binary64 beyond.
struct DiffAcc {
    float es = 0.f, ee = 0.f;  // largest error as s + e (two-sum parts)
    float ninf = 0.f, mn = 3.4e38f, mx = -3.4e38f;
    float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};  // e_1, e_2, n_1, n_2 (Neumaier)
    __device__ __forceinline__ void add(int k, float x)
    {
        const float t = __fadd_rn(s[k], x);
        c[k] = __fadd_rn(c[k], fabsf(s[k]) >= fabsf(x) ? __fadd_rn(__fsub_rn(s[k], t), x)
                                                       : __fadd_rn(__fsub_rn(x, t), s[k]));
        s[k] = t;
    }
    __device__ __forceinline__ void put(float f1, float f2)
    {
        // TwoSum(f1, -f2): d + r == f1 - f2 exactly
        const float d = __fadd_rn(f1, -f2);
        const float bv = __fsub_rn(d, f1);
        const float av = __fsub_rn(d, bv);
        const float r = __fadd_rn(__fsub_rn(f1, av), __fsub_rn(-f2, bv));
        const float a = fabsf(d);
        if (a > fabsf(es) || (a == fabsf(es) && fabs((double)d + r) > fabs((double)es + ee))) {
            es = d;
            ee = r;
        }
        const float n = fabsf(f2);
        ninf = fmaxf(ninf, n);
        mn = fminf(mn, f2);
        mx = fmaxf(mx, f2);
        // every term with its rounding error: |e| = a + sgn(d) r,
        // e^2 = a*a (+ fma residual) + 2 a sgn(d) r, n^2 = n*n (+ residual)
        const float sr = d >= 0.f ? r : -r;
        add(0, a);
        add(0, sr);
        const float a2 = __fmul_rn(a, a);
        add(1, a2);
        add(1, __fmaf_rn(a, a, -a2));
        add(1, __fmul_rn(2.f * a, sr));
        add(2, n);
        const float n2 = __fmul_rn(n, n);
        add(3, n2);
        add(3, __fmaf_rn(n, n, -n2));
    }
};

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int KIND, bool DIFF>
__global__ void __launch_bounds__(kNT, 1)
decode_kernel(const CzField *fields, int nfields, long long total_blocks, int shuffle, const uint8_t *base,
              const long long *rec_off, int *status, unsigned long long *queue, const float *diff_ref,
              double *diff_out, CzPlanes planes)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Shared s = carve(smem);
    __shared__ long long s_ticket, s_next;
    __shared__ int s_bad;
    // the next block's record, found by the last warp (s_pf_n < 0: none)
    __shared__ const uint8_t *s_pf_slot, *s_pf_q12;
    __shared__ int s_pf_n;
    constexpr int kPfWarp = kNT / 32 - 1;
    const int warp = threadIdx.x >> 5;
    // byte planes 1 and 2 of block b's record in the LZ4 input (or null)
    auto planes12 = [&](long long b, int nb) -> const uint8_t * {
        if (!planes.hole || !shuffle) return nullptr;
        const int c4 = (nb - kMaskBytes) / 4;
        const int4 h = planes.hole[b];
        return h.z > 0 && h.z == 2 * c4 && h.x == 4 + kMaskBytes + c4 ? planes.src + planes.src_off[b] + h.y
                                                                       : nullptr;
    };

    // tickets are taken one block ahead, so that the next block's record
    // can be brought into L2 while this one is transformed
    if (threadIdx.x == 0) s_next = (long long)atomicAdd(queue, 1ull);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            s_ticket = s_next;
            s_next = s_next < total_blocks ? (long long)atomicAdd(queue, 1ull) : total_blocks;
            s_bad = 0;
        }
        __syncthreads();
        const long long g = s_ticket;
        if (g >= total_blocks) break;
        const long long gn = s_next;
        const long long ron = warp == kPfWarp && gn < total_blocks ? rec_off[gn] : -1;  // used after the load
        const BlockRef ref = locate(fields, nfields, g);
        const long long ro = rec_off[g];
        const uint8_t *slot = base + (ro < 0 ? 0 : ro);
        const int nb = ro < 0 ? -1 : *reinterpret_cast<const int *>(slot);
        const bool size_ok = nb >= kMaskBytes && nb <= kMaxRecord + 4;
        // the payload into L2 while the mask is read and scanned (a no-op
        // when the previous block's pass already brought it)
        const uint8_t *q12 = size_ok ? planes12(g, nb) : nullptr;
        if (size_ok) prefetch_record(slot, nb, q12, threadIdx.x, kNT);
        // deserialize_bitset (WaveletCompressor.cpp:124-150)
        for (int i = threadIdx.x; i < kMaskBytes / 4; i += kNT)
            s.mask32[i] = size_ok ? reinterpret_cast<const uint32_t *>(slot + 4)[i] : 0u;
        __syncthreads();
        runs_from_mask(s);
        // the base case consumes exactly the 64 coarse survivors (:178-189)
        if (threadIdx.x < 16) {
            const int y = threadIdx.x & 3, z = threadIdx.x >> 2;
            if ((s.mask32[y + 32 * z] & 0xFu) != 0xFu) s_bad = 1;
        }
        __syncthreads();
        const int expected = scan_segments(s);
        const int payload = nb - kMaskBytes;
        int nel = payload / 4;
        if (nel - expected == 1) nel--;  // :247-250
        const bool ok = size_ok && nel == expected && !s_bad;
        if (threadIdx.x == 0) status[g] = ok ? 0 : -1;
        // ---- load (FullWaveletTransform.h:99-150): every survivor at its
        // place, read in stream order (consecutive across each warp), and
        // zeros at every other place (the runs cover the block); a bad
        // record leaves the block all zeros
        if (ok) {
            Payload pl;
            pl.p = slot + 4 + kMaskBytes;
            pl.c = payload / 4;
            pl.q = q12 ? q12 : pl.p + pl.c;  // planes 1 and 2
            pl.shuffle = shuffle != 0;
            load_survivors(s, expected, [&](int k) { return pl.get(k); });
        } else {
            for (int i = threadIdx.x; i < kBS3; i += kNT) s.sb[pidx(i & 31, (i >> 5) & 31, i >> 10)] = 0.f;
        }
        __syncthreads();
        // the last warp finds the next record while level 8 runs on the
        // first two warps
        if (warp == kPfWarp) {
            const int nbn = ron >= 0 ? *reinterpret_cast<const int *>(base + ron) : -1;
            const bool okn = nbn >= kMaskBytes && nbn <= kMaxRecord + 4;
            const uint8_t *qn = okn ? planes12(gn, nbn) : nullptr;
            if ((threadIdx.x & 31) == 0) {
                s_pf_slot = base + (ron < 0 ? 0 : ron);
                s_pf_q12 = qn;
                s_pf_n = okn ? nbn : -1;
            }
        }
        // ---- iwt: level 8 (x, z, y), level 16 (y, x, z), level 32 (z, y, x)
        sweep<8, 0, false, KIND>(s.sb);
        __syncthreads();
        sweep<8, 2, false, KIND>(s.sb);
        __syncthreads();
        sweep<8, 1, false, KIND>(s.sb);
        __syncthreads();
        // threads 256-511, idle during level 16, bring the next record into L2
        if (threadIdx.x >= 256 && s_pf_n > 0) prefetch_record(s_pf_slot, s_pf_n, s_pf_q12, threadIdx.x - 256, kNT - 256);
        sweep<16, 1, false, KIND>(s.sb);
        __syncthreads();
        sweep<16, 0, false, KIND>(s.sb);
        __syncthreads();
        sweep<16, 2, false, KIND>(s.sb);
        __syncthreads();
        sweep<32, 2, false, KIND>(s.sb);
        __syncthreads();
        sweep<32, 1, false, KIND>(s.sb);
        __syncthreads();
        // x lines: inverse, then straight to the field (copy_to, WaveletCompressor.h:73-82)
        float *out = const_cast<float *>(ref.f->data);
        DiffAcc acc;
        for (int l = threadIdx.x; l < 1024; l += kNT) {
            const int y = l & 31, z = l >> 5;
            float v[32];
            ld_line<32, 0>(s.sb, pidx(0, y, z), v);
            line_inv<32, KIND>(v);
            const size_t ro = row_offset(ref, y, z);
            float4 *dst = reinterpret_cast<float4 *>(out + ro);
#pragma unroll
            for (int k = 0; k < 8; ++k)
                __stcs(dst + k, make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
            if (DIFF) {
                const float4 *rr = reinterpret_cast<const float4 *>(diff_ref + ro);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const float4 q = __ldcs(rr + k);
                    acc.put(v[4 * k], q.x);
                    acc.put(v[4 * k + 1], q.y);
                    acc.put(v[4 * k + 2], q.z);
                    acc.put(v[4 * k + 3], q.w);
                }
            }
        }
        if (DIFF) {
            // block totals in binary64: maxima exact, sums of the compensated partials
            __shared__ double red[kNW][8];
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            double t[8];
            t[0] = warp_max(fabs((double)acc.es + acc.ee));
            t[1] = warp_max(acc.ninf);
            t[6] = -warp_max(-(double)acc.mn);
            t[7] = warp_max(acc.mx);
#pragma unroll
            for (int k = 0; k < 4; ++k) t[2 + k] = warp_sum((double)acc.s[k] + (double)acc.c[k]);
            if (lane == 0)
                for (int k = 0; k < 8; ++k) red[warp][k] = t[k];
            __syncthreads();
            if (threadIdx.x < 8) {
                const int k = threadIdx.x;
                double r = red[0][k];
                for (int w = 1; w < kNW; ++w) {
                    const double x = red[w][k];
                    r = (k == 0 || k == 1 || k == 7) ? fmax(r, x) : (k == 6 ? fmin(r, x) : r + x);
                }
                // e_1 n_1 e_2 n_2 order of the record: {e_inf, n_inf, e_1, e_2, n_1, n_2, min, max}
                diff_out[g * 8 + k] = r;
            }
        }
    }
}

// Totals over blocks, in block order: {e_inf, n_inf, e_1, e_2, n_1, n_2, min, max}.
// Field totals of the per-block statistics, in a fixed order: thread group j
// (of kDiffGroups) folds blocks j, j + kDiffGroups, ... in turn (four loads
// in flight, folded in block order), then the groups fold in order j = 0, 1,
// ... Deterministic for a given block count.
constexpr int kDiffGroups = 128;
__device__ __forceinline__ double diff_fold(int k, double r, double x)
{
    return (k == 0 || k == 1 || k == 7) ? fmax(r, x) : (k == 6 ? fmin(r, x) : r + x);
}
__global__ void __launch_bounds__(8 * kDiffGroups)
diff_total_kernel(const double *per_block, long long nblocks, double *total)
{
    __shared__ double part[kDiffGroups][8];
    __shared__ int have[kDiffGroups];
    const int k = threadIdx.x & 7, j = threadIdx.x >> 3;
    double r = 0.0;
    long long g = j;
    if (g < nblocks) {
        r = per_block[g * 8 + k];
        g += kDiffGroups;
    }
    for (; g + 3 * kDiffGroups < nblocks; g += 4 * kDiffGroups) {
        const double x0 = per_block[g * 8 + k], x1 = per_block[(g + kDiffGroups) * 8 + k];
        const double x2 = per_block[(g + 2 * kDiffGroups) * 8 + k], x3 = per_block[(g + 3 * kDiffGroups) * 8 + k];
        r = diff_fold(k, diff_fold(k, diff_fold(k, diff_fold(k, r, x0), x1), x2), x3);
    }
    for (; g < nblocks; g += kDiffGroups) r = diff_fold(k, r, per_block[g * 8 + k]);
    part[j][k] = r;
    if (k == 0) have[j] = j < nblocks;
    __syncthreads();
    if (j == 0) {
        double t = part[0][k];
        for (int i = 1; i < kDiffGroups; ++i)
            if (have[i]) t = diff_fold(k, t, part[i][k]);
        total[k] = t;
    }
}

}  // namespace cz

using namespace cz;

extern "C" int cz_codec_smem_bytes(void) { return kSmBytes; }

template <int KIND>
static cudaError_t launch_encode(const CzField *fields, int nfields, long long total_blocks, int zerobits,
                                 int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue, int grid,
                                 cudaStream_t st, int variant)
{
    auto k = variant == 1 ? encode_kernel<KIND, false> : encode_kernel<KIND, true>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    k<<<grid, kNT, kSmBytes, st>>>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue);
    return cudaGetLastError();
}

template <int KIND>
static cudaError_t launch_decode(const CzField *fields, int nfields, long long total_blocks, int shuffle,
                                 const uint8_t *base, const long long *rec_off, int *status,
                                 unsigned long long *queue, int grid, cudaStream_t st, const float *diff_ref,
                                 double *diff_out, CzPlanes planes)
{
    auto k = diff_ref ? decode_kernel<KIND, true> : decode_kernel<KIND, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    k<<<grid, kNT, kSmBytes, st>>>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, diff_ref,
                                   diff_out, planes);
    return cudaGetLastError();
}

cudaError_t cz_launch_encode(int wtype, const CzField *fields, int nfields, long long total_blocks, int zerobits,
                             int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue, int grid,
                             cudaStream_t st, int variant)
{
    switch (wkind(wtype)) {
    case 1:
        return launch_encode<1>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st,
                                variant);
    case 2:
        return launch_encode<2>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st,
                                variant);
    default:
        return launch_encode<3>(fields, nfields, total_blocks, zerobits, shuffle, stage, rec_bytes, queue, grid, st,
                                variant);
    }
}

cudaError_t cz_launch_decode(int wtype, const CzField *fields, int nfields, long long total_blocks, int shuffle,
                             const uint8_t *base, const long long *rec_off, int *status, unsigned long long *queue,
                             int grid, cudaStream_t st, const float *diff_ref, double *diff_out, CzPlanes planes)
{
    switch (wkind(wtype)) {
    case 1:
        return launch_decode<1>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st,
                                diff_ref, diff_out, planes);
    case 2:
        return launch_decode<2>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st,
                                diff_ref, diff_out, planes);
    default:
        return launch_decode<3>(fields, nfields, total_blocks, shuffle, base, rec_off, status, queue, grid, st,
                                diff_ref, diff_out, planes);
    }
}

cudaError_t cz_launch_diff_total(const double *per_block, long long nblocks, double *total, cudaStream_t st)
{
    if (nblocks < 1) return cudaErrorInvalidValue;
    diff_total_kernel<<<1, 8 * kDiffGroups, 0, st>>>(per_block, nblocks, total);
    return cudaGetLastError();
}
