// cz_device.cuh -- shared-memory block layout and device-side building blocks
// of the block codec kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cz_layout.cuh"
#include "cz_line.cuh"

namespace cz {

constexpr int kBS = 32;
constexpr int kBS3 = 32 * 32 * 32;
constexpr int kMaskBytes = 4096;                      // BITSETSIZE (WaveletCompressor.h:43)
constexpr int kMaxRecord = kMaskBytes + 4 * kBS3;     // BUFMAXSIZE (WaveletCompressor.h:44)
// One block's slot in the pre-LZ4 staging area: [int32 nbytes][record],
// rounded to 16 bytes and with 16 bytes of tail room for vector over-reads.
constexpr int kSlotBytes = ((4 + kMaxRecord + 15) / 16) * 16 + 16;

// A block lives in shared memory with x fastest and the x index XOR-swizzled
// by (y ^ z): lines along any axis, and the survivor-order gathers (whose
// lanes run along z at level 32), hit 32 distinct banks.
__device__ __forceinline__ int swz(int x, int y, int z) { return (z << 10) | (y << 5) | (x ^ ((y ^ z) & 31)); }

// Transform kinds, fixed per kernel instantiation: 1 interp, 2 lifted interp,
// 3 average-interpolating (the reference's wtype 0 and 3).
__host__ __device__ constexpr int wkind(int wtype) { return (wtype == 1 || wtype == 2) ? wtype : 3; }

template <int N, int KIND>
__device__ __forceinline__ void line_fwd(float (&v)[N])
{
    if (KIND == 3) fwd_avg<N>(v);
    else fwd_interp<N>(v, KIND == 2);
}
template <int N, int KIND>
__device__ __forceinline__ void line_inv(float (&v)[N])
{
    if (KIND == 3) inv_avg<N>(v);
    else inv_interp<N>(v, KIND == 2);
}

// One sweep of 1D transforms along AXIS (0 x, 1 y, 2 z) over the [0,N)^3
// corner, every thread taking whole lines. Lines are indexed so that
// consecutive lanes differ in the lowest non-line coordinate.
template <int N, int AXIS, bool FWD, int KIND, int NT>
__device__ __forceinline__ void sweep(float *sb)
{
    for (int line = threadIdx.x; line < N * N; line += NT) {
        const int a = line % N, c = line / N;
        float v[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int x = AXIS == 0 ? j : a;
            const int y = AXIS == 0 ? a : (AXIS == 1 ? j : c);
            const int z = AXIS == 2 ? j : c;
            v[j] = sb[swz(x, y, z)];
        }
        if (FWD) line_fwd<N, KIND>(v);
        else line_inv<N, KIND>(v);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int x = AXIS == 0 ? j : a;
            const int y = AXIS == 0 ? a : (AXIS == 1 ? j : c);
            const int z = AXIS == 2 ? j : c;
            sb[swz(x, y, z)] = v[j];
        }
    }
}

// The reference's level order expressed on mathematical axes
// (FullTransformEngine::fwt/iwt, FullWaveletTransform.h:44-56; axis orders
// derived in cz_layout.cuh).
template <int KIND, int NT>
__device__ __forceinline__ void forward_transform(float *sb)
{
    sweep<32, 0, true, KIND, NT>(sb);
    __syncthreads();
    sweep<32, 1, true, KIND, NT>(sb);
    __syncthreads();
    sweep<32, 2, true, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 2, true, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 0, true, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 1, true, KIND, NT>(sb);
    __syncthreads();
    sweep<8, 1, true, KIND, NT>(sb);
    __syncthreads();
    sweep<8, 2, true, KIND, NT>(sb);
    __syncthreads();
    sweep<8, 0, true, KIND, NT>(sb);
    __syncthreads();
}

template <int KIND, int NT>
__device__ __forceinline__ void inverse_transform(float *sb)
{
    sweep<8, 0, false, KIND, NT>(sb);
    __syncthreads();
    sweep<8, 2, false, KIND, NT>(sb);
    __syncthreads();
    sweep<8, 1, false, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 1, false, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 0, false, KIND, NT>(sb);
    __syncthreads();
    sweep<16, 2, false, KIND, NT>(sb);
    __syncthreads();
    sweep<32, 2, false, KIND, NT>(sb);
    __syncthreads();
    sweep<32, 1, false, KIND, NT>(sb);
    __syncthreads();
    sweep<32, 0, false, KIND, NT>(sb);
    __syncthreads();
}

// Physical smem index of the s-th survivor-order position.
__device__ __forceinline__ int swz_of_stream(int s, int &p)
{
    int px, py, pz, x, y, z;
    pos_of_stream(s, px, py, pz);
    phys_of_pos(px, py, pz, x, y, z);
    p = px + 32 * (py + 32 * pz);
    return swz(x, y, z);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace cz
