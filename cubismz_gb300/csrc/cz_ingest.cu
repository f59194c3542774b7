// cz_ingest.cu -- the layout of the reference's HDF5 tools next to the
// codec's x-fastest field.
//
// hdf2cz reads value (gx,gy,gz) from in[ch + nch*(gz + nz*(gy + ny*gx))]
// (z fastest, channels interleaved; Tools/Test_IO_Compressed.h:192-217) and
// cz2hdf writes decoded blocks back in the same order
// (Tools/cz2hdf.cpp:235-253, without _TRANSPOSE_DATA_). The codec works on
// out[gz][gy][gx] (x fastest). Both directions are an x<->z transpose per y
// plane: 32x32 tiles through shared memory (padded rows), reads coalesced
// along the source's fastest axis, writes along the destination's. Inputs in
// binary64 (the reference's precision=double builds) are rounded to the
// nearest binary32.
#include "cz_codec.h"

namespace cz {

constexpr int kTile = 32, kRows = 8;

// z-fastest (typed T, channel stride nch) -> x-fastest float
template <class T>
__global__ void __launch_bounds__(kTile *kRows)
from_zfastest_kernel(const T *__restrict__ in, int nch, int ch, int nx, int ny, int nz, float *__restrict__ out)
{
    __shared__ float tile[kTile][kTile + 1];
    const int z0 = blockIdx.x * kTile, x0 = blockIdx.y * kTile, y = blockIdx.z;
    const int tz = threadIdx.x, ty = threadIdx.y;
    // read: rows gx, columns gz (contiguous)
    for (int r = ty; r < kTile; r += kRows) {
        const int gx = x0 + r, gz = z0 + tz;
        if (gx < nx && gz < nz)
            tile[r][tz] = (float)in[(size_t)nch * ((size_t)gz + (size_t)nz * ((size_t)y + (size_t)ny * gx)) + ch];
    }
    __syncthreads();
    // write: rows gz, columns gx (contiguous)
    for (int r = ty; r < kTile; r += kRows) {
        const int gz = z0 + r, gx = x0 + tz;
        if (gx < nx && gz < nz) out[((size_t)gz * ny + y) * nx + gx] = tile[tz][r];
    }
}

// x-fastest float -> z-fastest float with channel stride nch
__global__ void __launch_bounds__(kTile *kRows)
to_zfastest_kernel(const float *__restrict__ in, int nx, int ny, int nz, int nch, int ch, float *__restrict__ out)
{
    __shared__ float tile[kTile][kTile + 1];
    const int x0 = blockIdx.x * kTile, z0 = blockIdx.y * kTile, y = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < kTile; r += kRows) {
        const int gz = z0 + r, gx = x0 + tx;
        if (gx < nx && gz < nz) tile[r][tx] = in[((size_t)gz * ny + y) * nx + gx];
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += kRows) {
        const int gx = x0 + r, gz = z0 + tx;
        if (gx < nx && gz < nz)
            out[(size_t)nch * ((size_t)gz + (size_t)nz * ((size_t)y + (size_t)ny * gx)) + ch] = tile[tx][r];
    }
}

}  // namespace cz

using namespace cz;

cudaError_t cz_launch_from_zfastest(const void *in, int bytes, int nch, int ch, int nx, int ny, int nz, float *out,
                                    cudaStream_t st)
{
    const dim3 grid((nz + kTile - 1) / kTile, (nx + kTile - 1) / kTile, ny), block(kTile, kRows);
    if (bytes == 8)
        from_zfastest_kernel<double><<<grid, block, 0, st>>>(static_cast<const double *>(in), nch, ch, nx, ny, nz, out);
    else
        from_zfastest_kernel<float><<<grid, block, 0, st>>>(static_cast<const float *>(in), nch, ch, nx, ny, nz, out);
    return cudaGetLastError();
}

cudaError_t cz_launch_to_zfastest(const float *in, int nx, int ny, int nz, int nch, int ch, float *out,
                                  cudaStream_t st)
{
    const dim3 grid((nx + kTile - 1) / kTile, (nz + kTile - 1) / kTile, ny), block(kTile, kRows);
    to_zfastest_kernel<<<grid, block, 0, st>>>(in, nx, ny, nz, nch, ch, out);
    return cudaGetLastError();
}
