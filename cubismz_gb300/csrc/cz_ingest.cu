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
//
// Single-channel arrays whose two transposed extents are multiples of the
// tile take the TMA path: tiles of 4 planes x 32 rows x 128 bytes move from
// HBM into shared memory by cp.async.bulk.tensor (128-byte swizzle, so that
// the column reads of the transpose hit at most 4 ways per bank; planes past
// the array come in zero-filled and are not stored), four tiles in flight
// per CTA on mbarriers, and every warp writes whole 128-byte rows of the
// destination. Each wait on an mbarrier is bounded; past the bound the
// CTA records an error, drains its copies in flight (bounded too) and
// returns, and the call reports the error.
#include <cuda.h>

#include <algorithm>

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

// ------------------------------------------------------------------ TMA path
constexpr int kStages = 4;
constexpr int kPlanes = 4;                                   // y planes per tile
constexpr int kTileBytes = kPlanes * 32 * 128;               // 16 KB
constexpr int kTmaSmem = kStages * kTileBytes + 1024;        // + alignment slack
constexpr long long kWaitLimit = 1ll << 22;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (long long i = 0; i < kWaitLimit; ++i) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, uint32_t bar,
                                            uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// Tile t of the source: planes y0..y0+3, 32 rows each (along the
// destination's fastest axis, r) of BC elements (along the source's fastest
// axis, c). Element (p, r, c) of the tile is written to
// out[(c0 + c)*sc + (y0 + p)*sy + r0 + r].
template <class T>
__global__ void __launch_bounds__(256)
tma_transpose_kernel(const __grid_constant__ CUtensorMap map, int ncb, int ny, int nrb, float *__restrict__ out,
                     long long sc, long long sy, int *err)
{
    constexpr int BC = 128 / (int)sizeof(T);  // elements per 128-byte row
    constexpr uint32_t kTile = kTileBytes;
    extern __shared__ unsigned char tma_smem[];
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tma_smem) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) unsigned long long bar[kStages];
    const int nyb = (ny + kPlanes - 1) / kPlanes;
    const long long ntiles = (long long)ncb * nyb * nrb;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto coords = [&](long long t, int &cb, int &y, int &rb) {
        cb = (int)(t % ncb);
        y = (int)((t / ncb) % nyb) * kPlanes;
        rb = (int)(t / ((long long)ncb * nyb));
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[s])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long long first = blockIdx.x, step = gridDim.x;
    if (threadIdx.x == 0)
        for (int s = 0; s < kStages; ++s) {
            const long long t = first + s * step;
            if (t >= ntiles) break;
            int cb, y, rb;
            coords(t, cb, y, rb);
            tma_load_3d(smem_u32(base + s * kTile), &map, cb * BC, rb * 32, y, smem_u32(&bar[s]), kTile);
        }
    bool ok = true;
    long long i = 0;
    for (long long t = first; t < ntiles; t += step, ++i) {
        const int s = (int)(i % kStages);
        const uint32_t parity = (uint32_t)((i / kStages) & 1);
        // the CTA leaves together if any thread's wait ran out
        if (!__syncthreads_and(mbar_wait(smem_u32(&bar[s]), parity) ? 1 : 0)) {
            ok = false;
            break;
        }
        int cb, y, rb;
        coords(t, cb, y, rb);
        const unsigned char *tile = base + s * kTile;
        const int np = min(kPlanes, ny - y);
        for (int pc = warp; pc < np * BC; pc += 8) {
            const int p = pc / BC, c = pc - p * BC;
            const int cbyte = c * (int)sizeof(T);
            const int off = p * 4096 + lane * 128 + ((((cbyte >> 4) ^ (lane & 7))) << 4) + (cbyte & 15);
            const T v = *reinterpret_cast<const T *>(tile + off);
            out[(long long)(cb * BC + c) * sc + (long long)(y + p) * sy + rb * 32 + lane] = (float)v;
        }
        __syncthreads();  // every thread is done with buf[s]
        if (threadIdx.x == 0) {
            const long long tn = t + kStages * step;
            if (tn < ntiles) {
                int cb2, y2, rb2;
                coords(tn, cb2, y2, rb2);
                tma_load_3d(smem_u32(base + s * kTile), &map, cb2 * BC, rb2 * 32, y2, smem_u32(&bar[s]), kTile);
            }
        }
    }
    if (!ok) {  // uniform across the CTA
        // record the error, then wait (bounded) for the copies still in flight
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            for (int k = 0; k < kStages; ++k) {
                const long long j = i + k;
                if (first + j * step >= ntiles) break;
                mbar_wait(smem_u32(&bar[j % kStages]), (uint32_t)((j / kStages) & 1));
            }
        }
        __syncthreads();
    }
}

}  // namespace cz

using namespace cz;

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Looked up once; the initialisation of a function-local static is
// thread-safe, so contexts on several host threads may reach it together.
EncodeTiled encode_tiled()
{
    static const EncodeTiled fn = []() -> EncodeTiled {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        const bool ok = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                                         &q) == cudaSuccess &&
                        q == cudaDriverEntryPointSuccess;
        cudaGetLastError();
        return ok ? reinterpret_cast<EncodeTiled>(p) : nullptr;
    }();
    return fn;
}

// The TMA transpose of a 3-D array (d0 fastest, then d1, d2) whose tiles are
// 128 bytes along d0 and 32 rows along d2; false if the map cannot be made
// (the caller then takes the plain kernel).
bool launch_tma(const void *in, int bytes, long long d0, long long d1, long long d2, float *out, long long sc,
                long long sy, int *err, cudaStream_t st)
{
    EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    const int bc = 128 / bytes;
    if (d0 % bc || d2 % 32 || reinterpret_cast<uintptr_t>(in) % 16) return false;
    // the map lists the rows' axis (d2) before the planes' (d1), so that a
    // box lands in shared memory as kPlanes whole 32-row tiles
    CUtensorMap map;
    const cuuint64_t dim[3] = {(cuuint64_t)d0, (cuuint64_t)d2, (cuuint64_t)d1};
    const cuuint64_t stride[2] = {(cuuint64_t)(d0 * d1 * bytes), (cuuint64_t)(d0 * bytes)};
    const cuuint32_t box[3] = {(cuuint32_t)bc, 32, (cuuint32_t)kPlanes}, es[3] = {1, 1, 1};
    if (stride[0] % 16 || stride[1] % 16) return false;
    if (enc(&map, bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
            const_cast<void *>(in), dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int ncb = (int)(d0 / bc), nrb = (int)(d2 / 32);
    const long long ntiles = (long long)ncb * ((d1 + kPlanes - 1) / kPlanes) * nrb;
    const int grid = (int)std::min<long long>(ntiles, (long long)sms * 3);
    auto k = bytes == 8 ? tma_transpose_kernel<double> : tma_transpose_kernel<float>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    k<<<grid, 256, kTmaSmem, st>>>(map, ncb, (int)d1, nrb, out, sc, sy, err);
    return true;
}

}  // namespace

cudaError_t cz_launch_from_zfastest(const void *in, int bytes, int nch, int ch, int nx, int ny, int nz, float *out,
                                    cudaStream_t st, int *err, bool *used_tma)
{
    if (used_tma) *used_tma = false;
    // source (z, y, x) z fastest; tile rows along x; out[z][y][x]
    if (err && nch == 1 && launch_tma(in, bytes, nz, ny, nx, out, (long long)ny * nx, nx, err, st)) {
        if (used_tma) *used_tma = true;
        return cudaGetLastError();
    }
    const dim3 grid((nz + kTile - 1) / kTile, (nx + kTile - 1) / kTile, ny), block(kTile, kRows);
    if (bytes == 8)
        from_zfastest_kernel<double><<<grid, block, 0, st>>>(static_cast<const double *>(in), nch, ch, nx, ny, nz, out);
    else
        from_zfastest_kernel<float><<<grid, block, 0, st>>>(static_cast<const float *>(in), nch, ch, nx, ny, nz, out);
    return cudaGetLastError();
}

cudaError_t cz_launch_to_zfastest(const float *in, int nx, int ny, int nz, int nch, int ch, float *out,
                                  cudaStream_t st, int *err, bool *used_tma)
{
    if (used_tma) *used_tma = false;
    // source (x, y, z) x fastest; tile rows along z; out[x][y][z]
    if (err && nch == 1 && launch_tma(in, 4, nx, ny, nz, out, (long long)ny * nz, nz, err, st)) {
        if (used_tma) *used_tma = true;
        return cudaGetLastError();
    }
    const dim3 grid((nx + kTile - 1) / kTile, (nz + kTile - 1) / kTile, ny), block(kTile, kRows);
    to_zfastest_kernel<<<grid, block, 0, st>>>(in, nx, ny, nz, nch, ch, out);
    return cudaGetLastError();
}
