// cz_refit.cu -- the inverse transform as a linear operator W, its adjoint
// W^T, and the least-squares refit of the retained coefficients.
//
// Interpolating wavelets are not orthogonal, so keeping the thresholded
// forward coefficients does not minimise the reconstruction error. With the
// significance mask M fixed by the plain path, the refit solves
//   min_c || x - W (M c) ||^2
// per block by CGLS (conjugate gradients on the normal equations, written on
// the residual), starting from the plain survivors. The record then carries
// the refit survivors under the same mask, so the stream layout, the chunking
// and the decoder are unchanged.
//
// W is the reference's iwt (FullWaveletTransform.h:51-56, sweep order of
// WaveletsOnInterval.h:249-276) evaluated in binary32 with its stencils as
// plain linear maps; W^T applies the transposed 1D operators in the reverse
// order. Both work on the kernels' block layout (cz_layout.cuh); the C-ABI
// entry points take and return coefficients in the reference's positional
// layout, the layout FullTransformEngine::fwt leaves in place.
#include "cz_block.cuh"
#include "cz_layout.cuh"

namespace cz {

// ------------------------------------------------------------ 1D operators
// Stencil coefficients are read into constexpr locals so that they fold
// into immediates (the coefficient tables are host-side constexpr arrays).
template <class S>
__device__ __forceinline__ float dot4(float a, float b, float c, float d)
{
    constexpr float k0 = S::c[0], k1 = S::c[1], k2 = S::c[2], k3 = S::c[3];
    return __fmaf_rn(k3, d, __fmaf_rn(k2, c, __fmaf_rn(k1, b, k0 * a)));
}
template <class S>
__device__ __forceinline__ float dot3(float a, float b, float c)
{
    constexpr float k0 = S::c[0], k1 = S::c[1], k2 = S::c[2];
    return __fmaf_rn(k2, c, __fmaf_rn(k1, b, k0 * a));
}
template <class S>
__device__ __forceinline__ void axpy4(float (&s)[16], int i, float g)  // s[i..i+3] += c * g
{
    constexpr float k0 = S::c[0], k1 = S::c[1], k2 = S::c[2], k3 = S::c[3];
    s[i] = __fmaf_rn(k0, g, s[i]);
    s[i + 1] = __fmaf_rn(k1, g, s[i + 1]);
    s[i + 2] = __fmaf_rn(k2, g, s[i + 2]);
    s[i + 3] = __fmaf_rn(k3, g, s[i + 3]);
}
template <class S>
__device__ __forceinline__ void axpy3(float (&s)[16], int i, float g)
{
    constexpr float k0 = S::c[0], k1 = S::c[1], k2 = S::c[2];
    s[i] = __fmaf_rn(k0, g, s[i]);
    s[i + 1] = __fmaf_rn(k1, g, s[i + 1]);
    s[i + 2] = __fmaf_rn(k2, g, s[i + 2]);
}

// Inverse line transform (WaveletsOnInterval.h:131-152, :181-198) as a
// linear map: [s | d] -> samples.
template <int N, int KIND>
__device__ __forceinline__ void lin_inv(float (&v)[N])
{
    constexpr int H = N / 2;
    float s[H], d[H];
#pragma unroll
    for (int i = 0; i < H; ++i) {
        d[i] = v[H + i];
        s[i] = KIND == 2 ? __fmaf_rn(-0.5f, d[i], v[i]) : v[i];
    }
    if (KIND != 3) {
        float o[H];
        o[0] = dot4<W1F>(s[0], s[1], s[2], s[3]);
#pragma unroll
        for (int i = 1; i < H - 2; ++i) o[i] = dot4<W1M>(s[i - 1], s[i], s[i + 1], s[i + 2]);
        o[H - 2] = dot4<W1O>(s[H - 4], s[H - 3], s[H - 2], s[H - 1]);
        o[H - 1] = dot4<W1L>(s[H - 4], s[H - 3], s[H - 2], s[H - 1]);
#pragma unroll
        for (int i = 0; i < H; ++i) {
            v[2 * i] = s[i];
            v[2 * i + 1] = o[i] + d[i];
        }
    } else {
        v[0] = dot3<P0F>(s[0], s[1], s[2]) - d[0];
        v[1] = dot3<P1F>(s[0], s[1], s[2]) + d[0];
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            v[2 * i] = dot3<P0M>(s[i - 1], s[i], s[i + 1]) - d[i];
            v[2 * i + 1] = dot3<P1M>(s[i - 1], s[i], s[i + 1]) + d[i];
        }
        v[N - 2] = dot3<P0L>(s[H - 3], s[H - 2], s[H - 1]) - d[H - 1];
        v[N - 1] = dot3<P1L>(s[H - 3], s[H - 2], s[H - 1]) + d[H - 1];
    }
}

// Its transpose: samples -> [s | d].
template <int N, int KIND>
__device__ __forceinline__ void lin_inv_t(float (&v)[N])
{
    constexpr int H = N / 2;
    float s[16], d[H];
    if (KIND != 3) {
#pragma unroll
        for (int i = 0; i < H; ++i) {
            s[i] = v[2 * i];
            d[i] = v[2 * i + 1];
        }
        axpy4<W1F>(s, 0, d[0]);
#pragma unroll
        for (int i = 1; i < H - 2; ++i) axpy4<W1M>(s, i - 1, d[i]);
        axpy4<W1O>(s, H - 4, d[H - 2]);
        axpy4<W1L>(s, H - 4, d[H - 1]);
#pragma unroll
        for (int i = 0; i < H; ++i) {
            v[i] = s[i];
            v[H + i] = KIND == 2 ? __fmaf_rn(-0.5f, s[i], d[i]) : d[i];
        }
    } else {
#pragma unroll
        for (int i = 0; i < H; ++i) {
            s[i] = 0.f;
            d[i] = v[2 * i + 1] - v[2 * i];
        }
        axpy3<P0F>(s, 0, v[0]);
        axpy3<P1F>(s, 0, v[1]);
#pragma unroll
        for (int i = 1; i < H - 1; ++i) {
            axpy3<P0M>(s, i - 1, v[2 * i]);
            axpy3<P1M>(s, i - 1, v[2 * i + 1]);
        }
        axpy3<P0L>(s, H - 3, v[N - 2]);
        axpy3<P1L>(s, H - 3, v[N - 1]);
#pragma unroll
        for (int i = 0; i < H; ++i) {
            v[i] = s[i];
            v[H + i] = d[i];
        }
    }
}

// ------------------------------------------------------------ 3D operators
template <int N, int AXIS, bool T, int KIND>
__device__ __forceinline__ void lsweep(float *sb)
{
    for (int l = threadIdx.x; l < N * N; l += kNT) {
        const int base = line_base<N, AXIS>(l);
        float v[N];
        ld_line<N, AXIS>(sb, base, v);
        if (T) lin_inv_t<N, KIND>(v);
        else lin_inv<N, KIND>(v);
        st_line<N, AXIS>(sb, base, v);
    }
    __syncthreads();
}

// W: level 8 (x, z, y), level 16 (y, x, z), level 32 (z, y, x) -- the decode
// kernel's order. Called and returns with the block synchronised.
template <int KIND>
__device__ __forceinline__ void w_apply(float *sb)
{
    lsweep<8, 0, false, KIND>(sb);
    lsweep<8, 2, false, KIND>(sb);
    lsweep<8, 1, false, KIND>(sb);
    lsweep<16, 1, false, KIND>(sb);
    lsweep<16, 0, false, KIND>(sb);
    lsweep<16, 2, false, KIND>(sb);
    lsweep<32, 2, false, KIND>(sb);
    lsweep<32, 1, false, KIND>(sb);
    lsweep<32, 0, false, KIND>(sb);
}
// W, returning this thread's part of ||W v||^2: the last sweep (x lines of
// level 32) sums the squares of the lines it writes.
template <int KIND>
__device__ __forceinline__ float w_apply_norm(float *sb)
{
    lsweep<8, 0, false, KIND>(sb);
    lsweep<8, 2, false, KIND>(sb);
    lsweep<8, 1, false, KIND>(sb);
    lsweep<16, 1, false, KIND>(sb);
    lsweep<16, 0, false, KIND>(sb);
    lsweep<16, 2, false, KIND>(sb);
    lsweep<32, 2, false, KIND>(sb);
    lsweep<32, 1, false, KIND>(sb);
    float acc = 0.f;
    for (int l = threadIdx.x; l < 32 * 32; l += kNT) {
        const int base = line_base<32, 0>(l);
        float v[32];
        ld_line<32, 0>(sb, base, v);
        lin_inv<32, KIND>(v);
        st_line<32, 0>(sb, base, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc = __fmaf_rn(v[j], v[j], acc);
    }
    __syncthreads();
    return acc;
}
template <int KIND>
__device__ __forceinline__ void wt_apply(float *sb)
{
    lsweep<32, 0, true, KIND>(sb);
    lsweep<32, 1, true, KIND>(sb);
    lsweep<32, 2, true, KIND>(sb);
    lsweep<16, 2, true, KIND>(sb);
    lsweep<16, 0, true, KIND>(sb);
    lsweep<16, 1, true, KIND>(sb);
    lsweep<8, 1, true, KIND>(sb);
    lsweep<8, 2, true, KIND>(sb);
    lsweep<8, 0, true, KIND>(sb);
}

// Dense element i of a block (x fastest) and its padded shared address.
__device__ __forceinline__ int pad_of(int i) { return pidx(i & 31, (i >> 5) & 31, i >> 10); }

// Block coefficient at positional index i <-> padded address of its
// physical (kernel-layout) place.
__device__ __forceinline__ int pad_of_pos(int i)
{
    int x, y, z;
    phys_of_pos(i & 31, (i >> 5) & 31, i >> 10, x, y, z);
    return pidx(x, y, z);
}

// Sum over the CTA (every thread gets it); `red` holds kNW doubles.
__device__ __forceinline__ double block_sum(double v, double *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
#pragma unroll
    for (int w = 0; w < kNW; ++w) t += red[w];
    __syncthreads();
    return t;
}

// ------------------------------------------------------------ dense kernels
template <int KIND>
__global__ void __launch_bounds__(kNT, 1) iwt_linear_kernel(const float *coef, float *out, long long nblocks)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *sb = reinterpret_cast<float *>(smem);
    for (long long g = blockIdx.x; g < nblocks; g += gridDim.x) {
        const float *src = coef + g * kBS3;
        for (int i = threadIdx.x; i < kBS3; i += kNT) sb[pad_of_pos(i)] = src[i];
        __syncthreads();
        w_apply<KIND>(sb);
        float *dst = out + g * kBS3;
        for (int i = threadIdx.x; i < kBS3; i += kNT) dst[i] = sb[pad_of(i)];
        __syncthreads();
    }
}

template <int KIND>
__global__ void __launch_bounds__(kNT, 1) iwt_adjoint_kernel(const float *in, float *coef, long long nblocks)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *sb = reinterpret_cast<float *>(smem);
    for (long long g = blockIdx.x; g < nblocks; g += gridDim.x) {
        const float *src = in + g * kBS3;
        for (int i = threadIdx.x; i < kBS3; i += kNT) sb[pad_of(i)] = src[i];
        __syncthreads();
        wt_apply<KIND>(sb);
        float *dst = coef + g * kBS3;
        for (int i = threadIdx.x; i < kBS3; i += kNT) dst[i] = sb[pad_of_pos(i)];
        __syncthreads();
    }
}

// ------------------------------------------------------------ refit
// Per block: the forward transform and thresholding of the encode kernel,
// CGLS on min ||x - W M c||^2 from the plain survivors, then the record.
// Each CTA keeps its block's iterates c, p (coefficients) and r (residual) in
// its own 3 x 128 KB of `scratch`; the block in shared memory carries W p,
// then r, then W^T r.
template <int KIND>
__global__ void __launch_bounds__(kNT, 1)
refit_kernel(const CzField *fields, int nfields, long long total_blocks, int zerobits, int shuffle, int iters,
             uint8_t *stage, int *rec_bytes, unsigned long long *queue, float *scratch)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Shared s = carve(smem);
    __shared__ long long s_ticket;
    __shared__ double red[kNW];
    const uint32_t zmask = zerobits > 0 ? ~((1u << zerobits) - 1u) : 0xffffffffu;
    float *Cv = scratch + (size_t)blockIdx.x * 3 * kBS3, *Pv = Cv + kBS3, *Rv = Pv + kBS3;
    float *sb = s.sb;

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_ticket = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        const long long g = s_ticket;
        if (g >= total_blocks) break;
        const BlockRef ref = locate(fields, nfields, g);
        const float eps = ref.f->eps;
        // ---- forward transform and masks (the encode kernel's sequence)
        for (int l = threadIdx.x; l < 1024; l += kNT) {
            const int y = l & 31, z = l >> 5;
            const float4 *row = reinterpret_cast<const float4 *>(ref.f->data + row_offset(ref, y, z));
            float v[32];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float4 q = __ldg(row + k);
                v[4 * k] = q.x;
                v[4 * k + 1] = q.y;
                v[4 * k + 2] = q.z;
                v[4 * k + 3] = q.w;
            }
            line_fwd<32, KIND>(v);
            st_line<32, 0>(sb, pidx(0, y, z), v);
        }
        __syncthreads();
        sweep<32, 1, true, KIND>(sb);
        __syncthreads();
        for (int l = threadIdx.x; l < 1024; l += kNT) {
            const int x = l & 31, y = l >> 5;
            const int base = pidx(x, y, 0);
            float v[32];
            ld_line<32, 2>(sb, base, v);
            line_fwd<32, KIND>(v);
            st_line<32, 2>(sb, base, v);
            emit32(s, x, y, keep_bits<32>(v, eps));
        }
        __syncthreads();
        sweep<16, 2, true, KIND>(sb);
        __syncthreads();
        sweep<16, 0, true, KIND>(sb);
        __syncthreads();
        if (threadIdx.x < 256) {
            const int x = threadIdx.x & 15, z = threadIdx.x >> 4;
            const int base = pidx(x, 0, z);
            float v[16];
            ld_line<16, 1>(sb, base, v);
            line_fwd<16, KIND>(v);
            st_line<16, 1>(sb, base, v);
            emit16(s, x, z, keep_bits<16>(v, eps));
        }
        __syncthreads();
        sweep<8, 1, true, KIND>(sb);
        __syncthreads();
        sweep<8, 2, true, KIND>(sb);
        __syncthreads();
        if (threadIdx.x < 64) {
            const int y = threadIdx.x & 7, z = threadIdx.x >> 3;
            const int base = pidx(0, y, z);
            float v[8];
            ld_line<8, 0>(sb, base, v);
            line_fwd<8, KIND>(v);
            st_line<8, 0>(sb, base, v);
            emit8(s, y, z, keep_bits<8>(v, eps));
        }
        __syncthreads();
        // The element passes below work on 4 consecutive elements (x
        // fastest) per thread and step: 16-byte loads and stores of the
        // iterates, several in flight per thread (the iterates live in L2).
        // Keep bits of elements i0 .. i0+3 (bit e for i0 + e).
        // The keep bits in kernel layout (word y + 32 z, bit x), built once
        // per block by warp votes into the emission stage, which is idle
        // until the record is written.
        uint32_t *km = reinterpret_cast<uint32_t *>(s.stage);
        for (int row = threadIdx.x >> 5; row < 1024; row += kNW) {
            const int x = threadIdx.x & 31, m = mask_index(x, row & 31, row >> 5);
            const unsigned w = __ballot_sync(0xffffffffu, (s.mask32[m >> 5] >> (m & 31)) & 1u);
            if (x == 0) km[row] = w;
        }
        __syncthreads();
        auto keep4 = [&](int i0) -> unsigned { return (km[i0 >> 5] >> (i0 & 31)) & 0xFu; };
        float4 *C4 = reinterpret_cast<float4 *>(Cv), *P4 = reinterpret_cast<float4 *>(Pv),
               *R4 = reinterpret_cast<float4 *>(Rv);
        constexpr int kV = kBS3 / 4;
        // ---- c0 = M c_full; r = x - W c0; s = M W^T r; p = s (also in sb)
#pragma unroll 4
        for (int j = threadIdx.x; j < kV; j += kNT) {
            const int i0 = 4 * j, a = pad_of(i0);
            const unsigned k = keep4(i0);
            float4 v;
            v.x = (k & 1u) ? sb[a] : 0.f;
            v.y = (k & 2u) ? sb[a + 1] : 0.f;
            v.z = (k & 4u) ? sb[a + 2] : 0.f;
            v.w = (k & 8u) ? sb[a + 3] : 0.f;
            sb[a] = v.x;
            sb[a + 1] = v.y;
            sb[a + 2] = v.z;
            sb[a + 3] = v.w;
            C4[j] = v;
        }
        __syncthreads();
        w_apply<KIND>(sb);
#pragma unroll 4
        for (int j = threadIdx.x; j < kV; j += kNT) {
            const int i0 = 4 * j, a = pad_of(i0);
            const float4 xv =
                __ldg(reinterpret_cast<const float4 *>(ref.f->data + row_offset(ref, (i0 >> 5) & 31, i0 >> 10)) +
                      ((i0 & 31) >> 2));
            float4 r;
            r.x = xv.x - sb[a];
            r.y = xv.y - sb[a + 1];
            r.z = xv.z - sb[a + 2];
            r.w = xv.w - sb[a + 3];
            R4[j] = r;
            sb[a] = r.x;
            sb[a + 1] = r.y;
            sb[a + 2] = r.z;
            sb[a + 3] = r.w;
        }
        __syncthreads();
        wt_apply<KIND>(sb);
        float acc = 0.f;
#pragma unroll 4
        for (int j = threadIdx.x; j < kV; j += kNT) {
            const int i0 = 4 * j, a = pad_of(i0);
            const unsigned k = keep4(i0);
            float4 v;
            v.x = (k & 1u) ? sb[a] : 0.f;
            v.y = (k & 2u) ? sb[a + 1] : 0.f;
            v.z = (k & 4u) ? sb[a + 2] : 0.f;
            v.w = (k & 8u) ? sb[a + 3] : 0.f;
            sb[a] = v.x;
            sb[a + 1] = v.y;
            sb[a + 2] = v.z;
            sb[a + 3] = v.w;
            P4[j] = v;
            acc = __fmaf_rn(v.x, v.x, __fmaf_rn(v.y, v.y, __fmaf_rn(v.z, v.z, __fmaf_rn(v.w, v.w, acc))));
        }
        double gamma = block_sum(acc, red);  // its barriers also order sb for W
        for (int it = 0; it < iters && gamma > 0.0; ++it) {
            // q = W p (sb holds p); ||q||^2 from the last sweep's lines
            acc = w_apply_norm<KIND>(sb);
            const double delta = block_sum(acc, red);
            if (!(delta > 0.0)) break;
            const float alpha = (float)(gamma / delta);
            // c += alpha p; r -= alpha q (sb gets r)
#pragma unroll 4
            for (int j = threadIdx.x; j < kV; j += kNT) {
                const int a = pad_of(4 * j);
                const float4 pv = P4[j];
                float4 cv = C4[j], rv = R4[j];
                cv.x = __fmaf_rn(alpha, pv.x, cv.x);
                cv.y = __fmaf_rn(alpha, pv.y, cv.y);
                cv.z = __fmaf_rn(alpha, pv.z, cv.z);
                cv.w = __fmaf_rn(alpha, pv.w, cv.w);
                rv.x = __fmaf_rn(-alpha, sb[a], rv.x);
                rv.y = __fmaf_rn(-alpha, sb[a + 1], rv.y);
                rv.z = __fmaf_rn(-alpha, sb[a + 2], rv.z);
                rv.w = __fmaf_rn(-alpha, sb[a + 3], rv.w);
                C4[j] = cv;
                R4[j] = rv;
                sb[a] = rv.x;
                sb[a + 1] = rv.y;
                sb[a + 2] = rv.z;
                sb[a + 3] = rv.w;
            }
            __syncthreads();
            // s = M W^T r; p = s + beta p (sb gets p for the next W)
            wt_apply<KIND>(sb);
            acc = 0.f;
#pragma unroll 4
            for (int j = threadIdx.x; j < kV; j += kNT) {
                const int i0 = 4 * j, a = pad_of(i0);
                const unsigned k = keep4(i0);
                const float v0 = (k & 1u) ? sb[a] : 0.f, v1 = (k & 2u) ? sb[a + 1] : 0.f,
                            v2 = (k & 4u) ? sb[a + 2] : 0.f, v3 = (k & 8u) ? sb[a + 3] : 0.f;
                sb[a] = v0;
                sb[a + 1] = v1;
                sb[a + 2] = v2;
                sb[a + 3] = v3;
                acc = __fmaf_rn(v0, v0, __fmaf_rn(v1, v1, __fmaf_rn(v2, v2, __fmaf_rn(v3, v3, acc))));
            }
            const double gnew = block_sum(acc, red);
            const float beta = (float)(gnew / gamma);
#pragma unroll 4
            for (int j = threadIdx.x; j < kV; j += kNT) {
                const int a = pad_of(4 * j);
                float4 pv = P4[j];
                pv.x = __fmaf_rn(beta, pv.x, sb[a]);
                pv.y = __fmaf_rn(beta, pv.y, sb[a + 1]);
                pv.z = __fmaf_rn(beta, pv.z, sb[a + 2]);
                pv.w = __fmaf_rn(beta, pv.w, sb[a + 3]);
                P4[j] = pv;
                sb[a] = pv.x;
                sb[a + 1] = pv.y;
                sb[a + 2] = pv.z;
                sb[a + 3] = pv.w;
            }
            gamma = gnew;
            __syncthreads();
        }
        // ---- the refit survivors go out under the plain mask
#pragma unroll 4
        for (int j = threadIdx.x; j < kBS3 / 4; j += kNT) {
            const int a = pad_of(4 * j);
            const float4 cv = reinterpret_cast<const float4 *>(Cv)[j];
            sb[a] = cv.x;
            sb[a + 1] = cv.y;
            sb[a + 2] = cv.z;
            sb[a + 3] = cv.w;
        }
        __syncthreads();
        emit_record(s, g, zmask, shuffle, stage, rec_bytes);
    }
}

}  // namespace cz

using namespace cz;

namespace {
template <class K>
cudaError_t prep(K kernel, int bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
constexpr int kDenseSmem = kPadFloats * 4;
}  // namespace

size_t cz_refit_scratch_floats(int grid) { return (size_t)grid * 3 * kBS3; }

cudaError_t cz_launch_iwt_linear(int wtype, const float *coef, float *out, long long nblocks, int grid, cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    cudaError_t e;
    switch (wkind(wtype)) {
    case 1:
        if ((e = prep(iwt_linear_kernel<1>, kDenseSmem)) != cudaSuccess) return e;
        iwt_linear_kernel<1><<<grid, kNT, kDenseSmem, st>>>(coef, out, nblocks);
        break;
    case 2:
        if ((e = prep(iwt_linear_kernel<2>, kDenseSmem)) != cudaSuccess) return e;
        iwt_linear_kernel<2><<<grid, kNT, kDenseSmem, st>>>(coef, out, nblocks);
        break;
    default:
        if ((e = prep(iwt_linear_kernel<3>, kDenseSmem)) != cudaSuccess) return e;
        iwt_linear_kernel<3><<<grid, kNT, kDenseSmem, st>>>(coef, out, nblocks);
    }
    return cudaGetLastError();
}

cudaError_t cz_launch_iwt_adjoint(int wtype, const float *in, float *coef, long long nblocks, int grid, cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    cudaError_t e;
    switch (wkind(wtype)) {
    case 1:
        if ((e = prep(iwt_adjoint_kernel<1>, kDenseSmem)) != cudaSuccess) return e;
        iwt_adjoint_kernel<1><<<grid, kNT, kDenseSmem, st>>>(in, coef, nblocks);
        break;
    case 2:
        if ((e = prep(iwt_adjoint_kernel<2>, kDenseSmem)) != cudaSuccess) return e;
        iwt_adjoint_kernel<2><<<grid, kNT, kDenseSmem, st>>>(in, coef, nblocks);
        break;
    default:
        if ((e = prep(iwt_adjoint_kernel<3>, kDenseSmem)) != cudaSuccess) return e;
        iwt_adjoint_kernel<3><<<grid, kNT, kDenseSmem, st>>>(in, coef, nblocks);
    }
    return cudaGetLastError();
}

cudaError_t cz_launch_refit(int wtype, const CzField *fields, int nfields, long long total_blocks, int zerobits,
                            int shuffle, int iters, uint8_t *stage, int *rec_bytes, unsigned long long *queue,
                            float *scratch, int grid, cudaStream_t st)
{
    if (total_blocks <= 0) return cudaSuccess;
    const int smem = cz_codec_smem_bytes();
    cudaError_t e;
    switch (wkind(wtype)) {
    case 1:
        if ((e = prep(refit_kernel<1>, smem)) != cudaSuccess) return e;
        refit_kernel<1><<<grid, kNT, smem, st>>>(fields, nfields, total_blocks, zerobits, shuffle, iters, stage,
                                                 rec_bytes, queue, scratch);
        break;
    case 2:
        if ((e = prep(refit_kernel<2>, smem)) != cudaSuccess) return e;
        refit_kernel<2><<<grid, kNT, smem, st>>>(fields, nfields, total_blocks, zerobits, shuffle, iters, stage,
                                                 rec_bytes, queue, scratch);
        break;
    default:
        if ((e = prep(refit_kernel<3>, smem)) != cudaSuccess) return e;
        refit_kernel<3><<<grid, kNT, smem, st>>>(fields, nfields, total_blocks, zerobits, shuffle, iters, stage,
                                                 rec_bytes, queue, scratch);
    }
    return cudaGetLastError();
}
