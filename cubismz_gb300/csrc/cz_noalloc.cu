// cz_noalloc.cu -- block compression that allocates no memory.
//
// Some callers cannot call cudaMalloc: applications that hand every byte of
// device memory to their own pool up front, and pipelines where an
// allocation would implicitly synchronise the device and stall work running
// beside the compressor. For them cz_blocks_compress_noalloc runs the same
// encode kernel as every other entry point, but its scratch memory (the
// block descriptor, the work-queue counter, the per-block record sizes and
// one staging slot per block) lives in the file-scope device array below,
// sized for CZ_NOALLOC_MAX_BLOCKS blocks (about 2.2 MB). Every GPU that
// loads the library holds that array until the process exits.
//
// Host code only ever passes the array's device address, obtained once per
// device with cudaGetSymbolAddress while that device is current (the
// symbol's name in host code is a host-side stand-in, not a device
// address). The first call on a device does this set-up, so it should come
// before any stream capture.
//
// All calls share the one array: it keeps the last call's contents, the
// counter and sizes are reset by every call, and calls that overlap on the
// GPU (different streams, or other threads) race on it.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/czgpu.h"
#include "cz_codec.h"
#include "cz_device.cuh"

namespace {

using cz::kSlotBytes;

constexpr int kMaxBlocks = CZ_NOALLOC_MAX_BLOCKS;
constexpr size_t kHdrBytes = 1024;  // descriptor, queue counter, record sizes
constexpr size_t kScratchBytes = kHdrBytes + (size_t)kMaxBlocks * kSlotBytes;
static_assert(sizeof(CzField) + 16 + 4 * kMaxBlocks <= kHdrBytes, "scratch header too small");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

struct Layout {
    CzField *field;
    unsigned long long *queue;
    int *rec_bytes;
    uint8_t *stage;
};

__host__ __device__ inline Layout layout(unsigned char *base)
{
    Layout l;
    l.field = reinterpret_cast<CzField *>(base);
    l.queue = reinterpret_cast<unsigned long long *>(base + 256);
    l.rec_bytes = reinterpret_cast<int *>(base + 512);
    l.stage = base + kHdrBytes;
    return l;
}

// Resets the queue counter and writes the descriptor: the blocks are a
// stack of 32^3 blocks along z (block g at d_blocks + g*32768).
__global__ void noalloc_init(unsigned char *base, const float *d_blocks, int nblocks, float eps)
{
    const Layout l = layout(base);
    *l.queue = 0ull;
    CzField f;
    f.data = d_blocks;
    f.nx = 32;
    f.ny = 32;
    f.nz = 32 * nblocks;
    f.eps = eps;
    f.block0 = 0;
    *l.field = f;
}

// Staging slot [int32 nbytes][record] -> caller's record buffer and size.
__global__ void noalloc_copy_out(unsigned char *base, int nblocks, uint8_t *d_records, int *d_nbytes)
{
    const Layout l = layout(base);
    const int g = blockIdx.x;
    if (g >= nblocks) return;
    const int nb = l.rec_bytes[g];
    const uint32_t *src = reinterpret_cast<const uint32_t *>(l.stage + (size_t)g * kSlotBytes + 4);
    uint32_t *dst = reinterpret_cast<uint32_t *>(d_records + (size_t)g * CZ_MAX_RECORD);
    for (int i = threadIdx.x; i < nb / 4; i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x == 0) d_nbytes[g] = nb;
}

// Device address of the scratch array for the current device.
int scratch_for_current(unsigned char **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return CZ_E_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return CZ_E_CUDA;
        }
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return CZ_OK;
}

}  // namespace

extern "C" int cz_blocks_compress_noalloc(const float *d_blocks, int nblocks, float eps, int wtype, int zerobits,
                                          int shuffle, uint8_t *d_records, int *d_nbytes, void *stream)
{
    if (!d_blocks || !d_records || !d_nbytes) return CZ_E_ARG;
    if (nblocks < 1 || nblocks > kMaxBlocks) return CZ_E_ARG;  // beyond the static scratch
    // the encode kernel reads blocks as float4 rows and the copy-out writes
    // records and sizes as 32-bit words: misaligned pointers are rejected
    // here instead of faulting on the device
    if ((reinterpret_cast<uintptr_t>(d_blocks) & 15u) || (reinterpret_cast<uintptr_t>(d_records) & 3u) ||
        (reinterpret_cast<uintptr_t>(d_nbytes) & 3u))
        return CZ_E_ARG;
    if (zerobits < 0 || zerobits > 31 || !(eps == eps)) return CZ_E_ARG;
    unsigned char *base = nullptr;
    const int rc = scratch_for_current(&base);
    if (rc != CZ_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Layout l = layout(base);
    noalloc_init<<<1, 1, 0, st>>>(base, d_blocks, nblocks, eps);
    if (cudaGetLastError() != cudaSuccess) return CZ_E_CUDA;
    int sms = 1;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = nblocks < sms ? nblocks : sms;
    if (cz_launch_encode(wtype, l.field, 1, nblocks, zerobits, shuffle ? 1 : 0, l.stage, l.rec_bytes, l.queue, grid,
                         st) != cudaSuccess) {
        cudaGetLastError();
        return CZ_E_CUDA;
    }
    noalloc_copy_out<<<nblocks, 256, 0, st>>>(base, nblocks, d_records, d_nbytes);
    if (cudaGetLastError() != cudaSuccess) return CZ_E_CUDA;
    return CZ_OK;
}
