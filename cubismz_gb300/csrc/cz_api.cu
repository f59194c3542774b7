// cz_api.cu -- the C-ABI of libczgpu.so (include/czgpu.h): context, device
// buffer management and the compress/decompress pipelines.
//
// Compress pipeline (one stream, no host round trip until the final size):
//   encode_kernel        fwt + threshold + mask + survivors -> block slots
//   chunk_setup          chunk geometry (blocks_per_chunk records per chunk)
//   pack_records         (blocks_per_chunk > 1) records back to back per chunk
//   lz4_encode_kernel    (encoder lz4) one warp per chunk
//   lz77 parse, deflate  (encoder zlib) one warp per chunk each
//   scan                 chunk offsets (replaces the writer's offset allocation)
//   gather               chunk payloads back to back
// Decompress pipeline: decode_setup, lz4_decode_kernel or inflate_kernel,
// record location, decode_kernel (load + iwt, optionally cz2diff's error
// sums) straight into the output field. cz_compress_to_image pipelines the
// compress steps over z-slabs behind the host-to-device copies.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/czgpu.h"
#include "cz_codec.h"
#include "cz_device.cuh"
#include "cz_format.h"

using namespace cz;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

constexpr long long lz4_bound_ll(long long n) { return n + n / 255 + 16; }
// zlib stream bound: header, Adler-32, and per block (every block but the
// last covers at least 1024 bytes; none is larger than its stored coding)
// at most 6 bytes beyond its data
constexpr long long zlib_bound_ll(long long n) { return n + 6 * (n / 1024 + 2) + 8; }
// DEFLATE parse records of a chunk (cz_launch_lz77_parse)
constexpr long long seq_bound_ll(long long n) { return 8 * (n / 4 + 2); }

}  // namespace

struct cz_ctx {
    int device = 0;
    int sms = 1;
    std::string err;
    DevBuf fields, stage, rec_bytes, chunk_in, in_off, in_len, blk_dst, lz_off, lz_out, lz_len, out_off, out_data,
        queue, status, flag, rec_off, dec, dec_off, dec_cap, dec_len, raw_off, chunk_rec, block_chunk, block_subid,
        tmp_field, tmp_in, refit, diff, zout, zoff, zlen, ierr, lz_hole;
    void *pin = nullptr;  // small pinned host scratch
    size_t pin_cap = 0;
    // geometry of the last compressed stream
    long long nblocks = 0;
    int nchunks = 0, bpc = 1;
    // stage timing
    bool timing = false;
    // LZ4 / LZ77 parse effort (cz_set_lz4_effort)
    int lz_effort = 1;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float stage_ms[3] = {0, 0, 0};
    // the pipelined host-buffer path: copy, LZ4 and gather streams, events per slab
    cudaStream_t s_copy = nullptr, s_gather = nullptr, s_comp = nullptr;
    std::vector<cudaStream_t> s_lz;
    std::vector<cudaEvent_t> ev_h2d, ev_enc, ev_lz;
    cudaEvent_t ev_join = nullptr;
};

namespace {

int fail(cz_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

#define CZ_CUDA(ctx, call)                                                                          \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(ctx, CZ_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int grow(cz_ctx *c, DevBuf &b, size_t bytes)
{
    if (bytes <= b.cap && b.p) return CZ_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    // 256 bytes of tail room: word-wise copies may read a few bytes past the end
    size_t want = bytes + 256;
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, CZ_E_NOMEM, "device allocation of " + std::to_string(want) + " bytes failed");
    }
    b.cap = want;
    return CZ_OK;
}

int grow_pin(cz_ctx *c, size_t bytes)
{
    if (bytes <= c->pin_cap && c->pin) return CZ_OK;
    if (c->pin) cudaFreeHost(c->pin);
    c->pin = nullptr;
    c->pin_cap = 0;
    if (cudaMallocHost(&c->pin, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, CZ_E_NOMEM, "pinned host allocation failed");
    }
    c->pin_cap = bytes;
    return CZ_OK;
}

#define CZ_TRY(x)                  \
    do {                           \
        const int r_ = (x);        \
        if (r_ != CZ_OK) return r_; \
    } while (0)

template <class T>
T *P(DevBuf &b)
{
    return reinterpret_cast<T *>(b.p);
}

int check_params(cz_ctx *c, const cz_params *p)
{
    if (!p) return fail(c, CZ_E_ARG, "params is NULL");
    if (p->zerobits < 0 || p->zerobits > 31) return fail(c, CZ_E_ARG, "zerobits must be in [0,31]");
    if (p->encoder != CZ_ENCODER_NONE && p->encoder != CZ_ENCODER_LZ4 && p->encoder != CZ_ENCODER_ZLIB)
        return fail(c, CZ_E_ARG, "encoder must be CZ_ENCODER_NONE, CZ_ENCODER_LZ4 or CZ_ENCODER_ZLIB");
    if (p->blocks_per_chunk < 1 || p->blocks_per_chunk > 64) return fail(c, CZ_E_ARG, "blocks_per_chunk must be in [1,64]");
    if (!(p->eps == p->eps)) return fail(c, CZ_E_ARG, "eps is NaN");
    return CZ_OK;
}

int check_dims(cz_ctx *c, int nx, int ny, int nz)
{
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx % 32 || ny % 32 || nz % 32)
        return fail(c, CZ_E_ARG, "field extents must be positive multiples of 32");
    return CZ_OK;
}

// Device fields are read and written as float4 rows: a field pointer must
// be 16-byte aligned (every cudaMalloc'd buffer is; an offset view may not
// be). Checked before any launch, so a bad pointer is an error, not a fault.
int check_align16(cz_ctx *c, const void *ptr, const char *what)
{
    if (reinterpret_cast<uintptr_t>(ptr) & 15u)
        return fail(c, CZ_E_ARG, std::string(what) + " must be 16-byte aligned");
    return CZ_OK;
}

int set_device(cz_ctx *c)
{
    CZ_CUDA(c, cudaSetDevice(c->device));
    return CZ_OK;
}

// stage marks k = 0..3 on the call's stream when timing is enabled
int mark(cz_ctx *c, int k, cudaStream_t st)
{
    if (!c->timing) return CZ_OK;
    if (!c->ev[k]) CZ_CUDA(c, cudaEventCreate(&c->ev[k]));
    CZ_CUDA(c, cudaEventRecord(c->ev[k], st));
    return CZ_OK;
}

// after the call's final synchronisation
void collect(cz_ctx *c)
{
    if (!c->timing) return;
    for (int k = 0; k < 3; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]) != cudaSuccess) {
            cudaGetLastError();
            ms = -1.f;
        }
        c->stage_ms[k] = ms;
    }
}

// The compress pipeline in three steps:
//   prepare  grows the context's buffers for the workload and uploads the
//            field descriptors (may allocate and copy);
//   enqueue  every device step on `st`, no allocation, no host wait (a CUDA
//            graph can capture it; sizes stay on the device);
//   finish   waits for the stream, reads the totals, fills *out.
struct Job {
    long long nblocks = 0;
    int nfields = 0, nchunks = 0, bpc = 1, lz_warps = 4, refit_iters = 0, enc_variant = 0;
    long long lz_slot = 0, z_slot = 0;  // per chunk: LZ4 output or DEFLATE parse; zlib output
    cz_params p{};
};

int prepare(cz_ctx *c, const std::vector<CzField> &fields, long long nblocks, const cz_params *p, int refit_iters,
            cudaStream_t st, Job &job)
{
    const int bpc = p->blocks_per_chunk;
    const long long nch_ll = (nblocks + bpc - 1) / bpc;
    if (nch_ll > 0x7fffffffLL) return fail(c, CZ_E_ARG, "too many chunks");
    job.nblocks = nblocks;
    job.nfields = (int)fields.size();
    job.nchunks = (int)nch_ll;
    job.bpc = bpc;
    job.p = *p;
    job.refit_iters = refit_iters;
    const long long chunk_max = (long long)bpc * kSlotBytes;
    const bool zlib = p->encoder == CZ_ENCODER_ZLIB;
    job.lz_slot = ((zlib ? seq_bound_ll(chunk_max) : lz4_bound_ll(chunk_max)) + 15) / 16 * 16;
    job.z_slot = zlib ? (zlib_bound_ll(chunk_max) + 16 + 15) / 16 * 16 : 0;
    const int nchunks = job.nchunks;
    CZ_TRY(grow(c, c->fields, sizeof(CzField) * fields.size()));
    CZ_TRY(grow(c, c->stage, (size_t)nblocks * kSlotBytes));
    CZ_TRY(grow(c, c->rec_bytes, sizeof(int) * nblocks));
    CZ_TRY(grow(c, c->in_off, sizeof(long long) * nchunks));
    CZ_TRY(grow(c, c->in_len, sizeof(int) * nchunks));
    CZ_TRY(grow(c, c->lz_off, sizeof(long long) * nchunks));
    CZ_TRY(grow(c, c->lz_len, sizeof(int) * nchunks));
    CZ_TRY(grow(c, c->out_off, sizeof(long long) * (nchunks + 1)));
    CZ_TRY(grow(c, c->raw_off, sizeof(long long) * (nchunks + 1)));
    CZ_TRY(grow(c, c->queue, 64));
    CZ_TRY(grow(c, c->flag, 64));
    if (bpc > 1) {
        CZ_TRY(grow(c, c->blk_dst, sizeof(long long) * nblocks));
        CZ_TRY(grow(c, c->chunk_in, (size_t)nchunks * bpc * kSlotBytes));
    }
    if (p->encoder != CZ_ENCODER_NONE) CZ_TRY(grow(c, c->lz_out, (size_t)nchunks * job.lz_slot));
    if (p->encoder == CZ_ENCODER_LZ4) CZ_TRY(grow(c, c->lz_hole, sizeof(int4) * (size_t)nchunks));
    if (zlib) {
        CZ_TRY(grow(c, c->zout, (size_t)nchunks * job.z_slot));
        CZ_TRY(grow(c, c->zoff, sizeof(long long) * nchunks));
        CZ_TRY(grow(c, c->zlen, sizeof(int) * nchunks));
    }
    // the gathered stream is bounded by the lossless bound of every chunk
    const size_t out_cap = (size_t)nchunks * (p->encoder == CZ_ENCODER_LZ4 ? job.lz_slot
                                                                           : (zlib ? job.z_slot : chunk_max));
    CZ_TRY(grow(c, c->out_data, out_cap));
    const int grid = (int)std::min<long long>(nblocks, c->sms);
    if (refit_iters > 0) CZ_TRY(grow(c, c->refit, sizeof(float) * cz_refit_scratch_floats(grid)));
    CZ_TRY(grow_pin(c, std::max<size_t>(4096, sizeof(CzField) * fields.size() + 64)));
    memcpy(c->pin, fields.data(), sizeof(CzField) * fields.size());
    // finish() reuses the pinned staging only after this copy (stream order)
    CZ_CUDA(c, cudaMemcpyAsync(c->fields.p, c->pin, sizeof(CzField) * fields.size(), cudaMemcpyHostToDevice, st));
    return CZ_OK;
}

int enqueue(cz_ctx *c, const Job &job, cudaStream_t st, bool marks)
{
    const cz_params *p = &job.p;
    const long long nblocks = job.nblocks;
    const int nchunks = job.nchunks, bpc = job.bpc;
    CZ_CUDA(c, cudaMemsetAsync(c->queue.p, 0, 64, st));
    CZ_CUDA(c, cudaMemsetAsync(c->flag.p, 0, 64, st));
    const int grid = (int)std::min<long long>(nblocks, c->sms);
    if (marks) CZ_TRY(mark(c, 0, st));
    if (job.refit_iters > 0)
        CZ_CUDA(c, cz_launch_refit(p->wtype, P<CzField>(c->fields), job.nfields, nblocks, p->zerobits,
                                   p->shuffle ? 1 : 0, job.refit_iters, P<uint8_t>(c->stage), P<int>(c->rec_bytes),
                                   P<unsigned long long>(c->queue), P<float>(c->refit), grid, st));
    else
        CZ_CUDA(c, cz_launch_encode(p->wtype, P<CzField>(c->fields), job.nfields, nblocks, p->zerobits,
                                    p->shuffle ? 1 : 0, P<uint8_t>(c->stage), P<int>(c->rec_bytes),
                                    P<unsigned long long>(c->queue), grid, st, job.enc_variant));
    if (marks) CZ_TRY(mark(c, 1, st));
    CZ_CUDA(c, cz_launch_chunk_setup(bpc, nblocks, nchunks, P<int>(c->rec_bytes), P<long long>(c->in_off),
                                     P<int>(c->in_len), bpc > 1 ? P<long long>(c->blk_dst) : nullptr,
                                     P<long long>(c->lz_off), job.lz_slot, st));
    const uint8_t *chunk_src = P<uint8_t>(c->stage);
    if (bpc > 1) {
        CZ_CUDA(c, cz_launch_pack_records(P<uint8_t>(c->stage), P<int>(c->rec_bytes), nblocks,
                                          P<long long>(c->blk_dst), P<uint8_t>(c->chunk_in), st));
        chunk_src = P<uint8_t>(c->chunk_in);
    }
    CZ_CUDA(c, cz_launch_scan(P<int>(c->in_len), nchunks, P<long long>(c->raw_off), st));
    const uint8_t *gsrc = chunk_src;
    const long long *gsrc_off = P<long long>(c->in_off);
    const int *glen = P<int>(c->in_len);
    if (p->encoder == CZ_ENCODER_LZ4) {
        const int per = job.lz_warps;
        const int lzgrid = std::max(1, std::min((nchunks + per - 1) / per, c->sms * (32 / per)));
        // the records' incompressible planes are left to the gather (hole)
        CZ_CUDA(c, cz_launch_lz4_encode(chunk_src, P<long long>(c->in_off), P<int>(c->in_len), nchunks,
                                        P<uint8_t>(c->lz_out), P<long long>(c->lz_off), P<int>(c->lz_len),
                                        p->shuffle ? 1 : 0, per, lzgrid, st, P<int4>(c->lz_hole), c->lz_effort));
        CZ_CUDA(c, cz_launch_neg_reduce(P<int>(c->lz_len), nchunks, P<int>(c->flag), st));
        gsrc = P<uint8_t>(c->lz_out);
        gsrc_off = P<long long>(c->lz_off);
        glen = P<int>(c->lz_len);
    } else if (p->encoder == CZ_ENCODER_ZLIB) {
        const int pgrid = std::max(1, std::min((nchunks + 3) / 4, c->sms * 8));
        CZ_CUDA(c, cz_launch_lz77_parse(chunk_src, P<long long>(c->in_off), P<int>(c->in_len), nchunks,
                                        P<uint8_t>(c->lz_out), P<long long>(c->lz_off), P<int>(c->lz_len),
                                        p->shuffle ? 1 : 0, pgrid, st, c->lz_effort));
        CZ_CUDA(c, cz_launch_deflate(chunk_src, P<long long>(c->in_off), P<int>(c->in_len), P<uint8_t>(c->lz_out),
                                     P<long long>(c->lz_off), P<int>(c->lz_len), nchunks, p->shuffle ? 1 : 0,
                                     P<uint8_t>(c->zout),
                                     job.z_slot, P<long long>(c->zoff), P<int>(c->zlen),
                                     std::max(1, std::min((nchunks + 3) / 4, c->sms * 5)), st));
        CZ_CUDA(c, cz_launch_neg_reduce(P<int>(c->zlen), nchunks, P<int>(c->flag), st));
        gsrc = P<uint8_t>(c->zout);
        gsrc_off = P<long long>(c->zoff);
        glen = P<int>(c->zlen);
    }
    if (marks) CZ_TRY(mark(c, 2, st));
    CZ_CUDA(c, cz_launch_scan(glen, nchunks, P<long long>(c->out_off), st));
    const bool holes = p->encoder == CZ_ENCODER_LZ4;
    CZ_CUDA(c, cz_launch_gather(gsrc, gsrc_off, glen, nchunks, P<uint8_t>(c->out_data), P<long long>(c->out_off), st,
                                holes ? P<int4>(c->lz_hole) : nullptr, chunk_src, P<long long>(c->in_off)));
    if (marks) CZ_TRY(mark(c, 3, st));
    return CZ_OK;
}

int finish(cz_ctx *c, const Job &job, cudaStream_t st, cz_stream *out)
{
    long long *h = reinterpret_cast<long long *>(c->pin);
    const int nchunks = job.nchunks;
    CZ_CUDA(c, cudaMemcpyAsync(&h[0], P<long long>(c->out_off) + nchunks, 8, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaMemcpyAsync(&h[1], P<long long>(c->raw_off) + nchunks, 8, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaMemcpyAsync(&h[2], c->flag.p, 4, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    if (reinterpret_cast<int *>(&h[2])[0] != 0)
        return fail(c, CZ_E_CUDA, "lossless encoder output exceeded its bound");
    c->nblocks = job.nblocks;
    c->nchunks = nchunks;
    c->bpc = job.bpc;
    out->data = P<uint8_t>(c->out_data);
    out->data_bytes = h[0];
    out->chunk_offsets = P<long long>(c->out_off);
    out->nchunks = nchunks;
    out->nblocks = job.nblocks;
    out->raw_bytes = h[1];
    return CZ_OK;
}

// The whole pipeline for descriptors in host memory; returns after the total
// size is known (one small device-to-host copy).
int compress_fields(cz_ctx *c, const std::vector<CzField> &fields, long long nblocks, const cz_params *p,
                    cudaStream_t st, cz_stream *out, int refit_iters = 0)
{
    Job job;
    CZ_TRY(prepare(c, fields, nblocks, p, refit_iters, st, job));
    CZ_TRY(enqueue(c, job, st, true));
    const int rc = finish(c, job, st, out);
    collect(c);
    return rc;
}

// Decompress pipeline for a field whose records sit in chunks of bpc
// consecutive blocks, or (block_chunk != NULL) with an explicit
// block -> (chunk, subid) map (files written by other writers).
int decompress_fields(cz_ctx *c, const std::vector<CzField> &fields, long long nblocks, const uint8_t *d_data,
                      const long long *d_off, int nchunks, int encoder, int wtype, int shuffle, int bpc,
                      const int *h_block_chunk, const int *h_block_subid, int maxsub, cudaStream_t st,
                      const float *diff_ref = nullptr, double *h_stats = nullptr)
{
    const int per_chunk = h_block_chunk ? maxsub : bpc;
    if (diff_ref) CZ_TRY(grow(c, c->diff, sizeof(double) * (8 * (size_t)nblocks + 8)));
    const long long dcap = ((long long)per_chunk * (4 + kMaxRecord) + 15) / 16 * 16;
    CZ_TRY(grow(c, c->fields, sizeof(CzField) * fields.size()));
    CZ_TRY(grow(c, c->in_len, sizeof(int) * nchunks));
    CZ_TRY(grow(c, c->dec_off, sizeof(long long) * nchunks));
    CZ_TRY(grow(c, c->dec_cap, sizeof(int) * nchunks));
    CZ_TRY(grow(c, c->dec_len, sizeof(int) * nchunks));
    CZ_TRY(grow(c, c->rec_off, sizeof(long long) * nblocks));
    CZ_TRY(grow(c, c->status, sizeof(int) * nblocks));
    CZ_TRY(grow(c, c->queue, 64));
    CZ_TRY(grow(c, c->flag, 64));
    if (encoder != CZ_ENCODER_NONE) CZ_TRY(grow(c, c->dec, (size_t)nchunks * dcap));
    // pinned scratch: [fields | flag (64 B) | block map]
    const size_t pin_fields = (sizeof(CzField) * fields.size() + 63) / 64 * 64;
    const size_t map_bytes = h_block_chunk ? sizeof(int) * 2 * nblocks : 0;
    CZ_TRY(grow_pin(c, std::max<size_t>(4096, pin_fields + 64 + map_bytes)));
    memcpy(c->pin, fields.data(), sizeof(CzField) * fields.size());
    CZ_CUDA(c, cudaMemcpyAsync(c->fields.p, c->pin, sizeof(CzField) * fields.size(), cudaMemcpyHostToDevice, st));
    CZ_CUDA(c, cudaMemsetAsync(c->queue.p, 0, 64, st));
    CZ_CUDA(c, cudaMemsetAsync(c->flag.p, 0, 64, st));
    const int raw = encoder == CZ_ENCODER_NONE;
    CZ_TRY(mark(c, 0, st));
    CZ_CUDA(c, cz_launch_decode_setup(nchunks, d_off, P<int>(c->in_len), P<long long>(c->dec_off), P<int>(c->dec_cap),
                                      dcap, raw, st));
    const uint8_t *base = d_data;
    const int *dlen = P<int>(c->in_len);
    // one shuffled record per chunk, blocks in chunk order: the LZ4 decoder
    // may leave the records' byte planes 1 and 2 in its input, where the
    // decode kernel reads them
    const bool planes_in_input = bpc == 1 && shuffle && !h_block_chunk && (long long)nchunks == nblocks;
    CzPlanes planes;
    if (encoder == CZ_ENCODER_ZLIB) {
        CZ_CUDA(c, cz_launch_inflate(d_data, d_off, P<int>(c->in_len), nchunks, P<uint8_t>(c->dec),
                                     P<long long>(c->dec_off), P<int>(c->dec_cap), P<int>(c->dec_len),
                                     std::min(nchunks, c->sms * 32), st));
        base = P<uint8_t>(c->dec);
        dlen = P<int>(c->dec_len);
    } else if (!raw) {
        const int lzgrid = std::max(1, std::min((nchunks + 3) / 4, c->sms * 8));
        if (planes_in_input) {
            CZ_TRY(grow(c, c->lz_hole, sizeof(int4) * (size_t)nchunks));
            planes = CzPlanes{P<int4>(c->lz_hole), d_data, d_off};
        }
        CZ_CUDA(c, cz_launch_lz4_decode(d_data, d_off, P<int>(c->in_len), nchunks, P<uint8_t>(c->dec),
                                        P<long long>(c->dec_off), P<int>(c->dec_cap), P<int>(c->dec_len), lzgrid, st,
                                        planes_in_input ? P<int4>(c->lz_hole) : nullptr));
        base = P<uint8_t>(c->dec);
        dlen = P<int>(c->dec_len);
    }
    CZ_TRY(mark(c, 1, st));
    if (h_block_chunk) {
        CZ_TRY(grow(c, c->chunk_rec, sizeof(long long) * (size_t)nchunks * maxsub));
        CZ_TRY(grow(c, c->block_chunk, sizeof(int) * nblocks));
        CZ_TRY(grow(c, c->block_subid, sizeof(int) * nblocks));
        int *hp = reinterpret_cast<int *>(reinterpret_cast<char *>(c->pin) + pin_fields + 64);
        memcpy(hp, h_block_chunk, sizeof(int) * nblocks);
        memcpy(hp + nblocks, h_block_subid, sizeof(int) * nblocks);
        CZ_CUDA(c, cudaMemcpyAsync(c->block_chunk.p, hp, sizeof(int) * nblocks, cudaMemcpyHostToDevice, st));
        CZ_CUDA(c, cudaMemcpyAsync(c->block_subid.p, hp + nblocks, sizeof(int) * nblocks, cudaMemcpyHostToDevice, st));
        const long long *cbase = raw ? d_off : P<long long>(c->dec_off);
        CZ_CUDA(c, cz_launch_chunk_records(nchunks, maxsub, cbase, dlen, base, P<long long>(c->chunk_rec), st));
        CZ_CUDA(c, cz_launch_map_blocks(nblocks, nchunks, maxsub, P<int>(c->block_chunk), P<int>(c->block_subid),
                                        P<long long>(c->chunk_rec), P<long long>(c->rec_off), st));
    } else {
        const long long *cbase = raw ? d_off : P<long long>(c->dec_off);
        CZ_CUDA(c, cz_launch_locate_records(bpc, nblocks, nchunks, cbase, dlen, P<long long>(c->rec_off),
                                            P<int>(c->status), base, st));
    }
    const int grid = (int)std::min<long long>(nblocks, c->sms);
    CZ_TRY(mark(c, 2, st));
    double *per_block = diff_ref ? P<double>(c->diff) : nullptr;
    CZ_CUDA(c, cz_launch_decode(wtype, P<CzField>(c->fields), (int)fields.size(), nblocks, shuffle ? 1 : 0, base,
                                P<long long>(c->rec_off), P<int>(c->status), P<unsigned long long>(c->queue), grid,
                                st, diff_ref, per_block, planes));
    if (diff_ref) CZ_CUDA(c, cz_launch_diff_total(per_block, nblocks, per_block + 8 * nblocks, st));
    CZ_TRY(mark(c, 3, st));
    CZ_CUDA(c, cz_launch_status_reduce(P<int>(c->status), nblocks, P<int>(c->flag), st));
    int *hflag = reinterpret_cast<int *>(reinterpret_cast<char *>(c->pin) + pin_fields);
    CZ_CUDA(c, cudaMemcpyAsync(hflag, c->flag.p, 4, cudaMemcpyDeviceToHost, st));
    if (diff_ref) CZ_CUDA(c, cudaMemcpyAsync(h_stats, per_block + 8 * nblocks, 64, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    collect(c);
    if (*hflag != 0) return fail(c, CZ_E_CORRUPT, "malformed chunk or record in the compressed stream");
    return CZ_OK;
}

}  // namespace

extern "C" {

int cz_create(int device, cz_ctx **out)
{
    if (!out) return CZ_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return CZ_E_CUDA;
    }
    cz_ctx *c = new cz_ctx;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return CZ_E_CUDA;
    }
    *out = c;
    return CZ_OK;
}

int cz_destroy(cz_ctx *c)
{
    if (!c) return CZ_OK;
    cudaSetDevice(c->device);
    DevBuf *all[] = {&c->ierr, &c->zout, &c->zoff, &c->zlen, &c->diff, &c->refit, &c->fields,  &c->stage,   &c->rec_bytes, &c->chunk_in,  &c->in_off,      &c->in_len,
                     &c->blk_dst, &c->lz_off,  &c->lz_out,    &c->lz_len,    &c->out_off,     &c->out_data,
                     &c->queue,   &c->status,  &c->flag,      &c->rec_off,   &c->dec,         &c->dec_off,
                     &c->dec_cap, &c->dec_len, &c->raw_off,   &c->chunk_rec, &c->block_chunk, &c->block_subid,
                     &c->tmp_field, &c->tmp_in, &c->lz_hole};
    for (DevBuf *b : all)
        if (b->p) cudaFree(b->p);
    for (cudaEvent_t e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto *v : {&c->ev_h2d, &c->ev_enc, &c->ev_lz})
        for (cudaEvent_t e : *v) cudaEventDestroy(e);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    for (cudaStream_t s : c->s_lz) cudaStreamDestroy(s);
    if (c->s_copy) cudaStreamDestroy(c->s_copy);
    if (c->s_gather) cudaStreamDestroy(c->s_gather);
    if (c->s_comp) cudaStreamDestroy(c->s_comp);
    if (c->pin) cudaFreeHost(c->pin);
    delete c;
    return CZ_OK;
}

const char *cz_last_error(cz_ctx *c) { return c ? c->err.c_str() : "no context"; }

int cz_set_timing(cz_ctx *c, int on)
{
    if (!c) return CZ_E_ARG;
    c->timing = on != 0;
    return CZ_OK;
}

int cz_set_lz4_effort(cz_ctx *c, int effort)
{
    if (!c || effort < 0 || effort > 2) return fail(c, CZ_E_ARG, "LZ4 effort must be 0, 1 or 2");
    c->lz_effort = effort;
    return CZ_OK;
}

int cz_stage_times(cz_ctx *c, float *ms, int n)
{
    if (!c || !ms || n < 0) return CZ_E_ARG;
    const int k = n < 3 ? n : 3;
    for (int i = 0; i < k; ++i) ms[i] = c->stage_ms[i];
    return k;
}

int cz_field_compress(cz_ctx *c, const float *d_field, int nx, int ny, int nz, const cz_params *p, void *stream,
                      cz_stream *out)
{
    if (!c || !d_field || !out) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(check_params(c, p));
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(check_align16(c, d_field, "d_field"));
    CZ_TRY(set_device(c));
    const long long nblocks = (long long)(nx / 32) * (ny / 32) * (nz / 32);
    std::vector<CzField> f(1);
    f[0] = CzField{d_field, nx, ny, nz, p->eps, 0};
    return compress_fields(c, f, nblocks, p, (cudaStream_t)stream, out);
}

int cz_refit(cz_ctx *c, const float *d_field, int nx, int ny, int nz, const cz_params *p, int iters, void *stream,
             cz_stream *out)
{
    if (!c || !d_field || !out) return fail(c, CZ_E_ARG, "NULL argument");
    if (iters < 1 || iters > 1000) return fail(c, CZ_E_ARG, "refit iterations out of range [1, 1000]");
    CZ_TRY(check_params(c, p));
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(check_align16(c, d_field, "d_field"));
    CZ_TRY(set_device(c));
    const long long nblocks = (long long)(nx / 32) * (ny / 32) * (nz / 32);
    std::vector<CzField> f(1);
    f[0] = CzField{d_field, nx, ny, nz, p->eps, 0};
    return compress_fields(c, f, nblocks, p, (cudaStream_t)stream, out, iters);
}

int cz_iwt_linear(cz_ctx *c, const float *d_coef, long long nblocks, int wtype, float *d_blocks, void *stream)
{
    if (!c || !d_coef || !d_blocks || nblocks < 0) return fail(c, CZ_E_ARG, "bad arguments");
    CZ_TRY(set_device(c));
    const int grid = (int)std::max<long long>(1, std::min<long long>(nblocks, c->sms));
    CZ_CUDA(c, cz_launch_iwt_linear(wtype, d_coef, d_blocks, nblocks, grid, (cudaStream_t)stream));
    return CZ_OK;
}

int cz_iwt_adjoint(cz_ctx *c, const float *d_blocks, long long nblocks, int wtype, float *d_coef, void *stream)
{
    if (!c || !d_coef || !d_blocks || nblocks < 0) return fail(c, CZ_E_ARG, "bad arguments");
    CZ_TRY(set_device(c));
    const int grid = (int)std::max<long long>(1, std::min<long long>(nblocks, c->sms));
    CZ_CUDA(c, cz_launch_iwt_adjoint(wtype, d_blocks, d_coef, nblocks, grid, (cudaStream_t)stream));
    return CZ_OK;
}

int cz_stream_copy(cz_ctx *c, const cz_stream *s, uint8_t *d_data, long long *d_off, void *stream)
{
    if (!c || !s) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(set_device(c));
    cudaStream_t st = (cudaStream_t)stream;
    long long base = 0;
    CZ_CUDA(c, cudaMemcpyAsync(&base, s->chunk_offsets, 8, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    if (d_data && s->data_bytes > 0)
        CZ_CUDA(c, cudaMemcpyAsync(d_data, s->data + base, (size_t)s->data_bytes, cudaMemcpyDeviceToDevice, st));
    if (d_off) {
        CZ_CUDA(c, cudaMemcpyAsync(d_off, s->chunk_offsets, sizeof(long long) * (s->nchunks + 1),
                                   cudaMemcpyDeviceToDevice, st));
        if (base) CZ_CUDA(c, cz_launch_rebase(d_off, s->nchunks + 1, base, st));
    }
    return CZ_OK;
}

int cz_field_decompress(cz_ctx *c, const uint8_t *d_data, const long long *d_off, int nchunks, int nx, int ny, int nz,
                        const cz_params *p, void *stream, float *d_field)
{
    if (!c || !d_data || !d_off || !d_field) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(check_params(c, p));
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(check_align16(c, d_field, "d_field"));
    CZ_TRY(set_device(c));
    const long long nblocks = (long long)(nx / 32) * (ny / 32) * (nz / 32);
    const int bpc = p->blocks_per_chunk;
    if ((long long)nchunks != (nblocks + bpc - 1) / bpc) return fail(c, CZ_E_ARG, "chunk count does not match the field");
    std::vector<CzField> f(1);
    f[0] = CzField{d_field, nx, ny, nz, p->eps, 0};
    return decompress_fields(c, f, nblocks, d_data, d_off, nchunks, p->encoder, p->wtype, p->shuffle, bpc, nullptr,
                             nullptr, 0, (cudaStream_t)stream);
}

int cz_field_diff(cz_ctx *c, const uint8_t *d_data, const long long *d_off, int nchunks, int nx, int ny, int nz,
                  const cz_params *p, const float *d_ref, void *stream, float *d_field, double *stats)
{
    if (!c || !d_data || !d_off || !d_ref || !stats) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(check_params(c, p));
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(check_align16(c, d_ref, "d_ref"));
    if (d_field) CZ_TRY(check_align16(c, d_field, "d_field"));
    CZ_TRY(set_device(c));
    const long long nblocks = (long long)(nx / 32) * (ny / 32) * (nz / 32);
    const int bpc = p->blocks_per_chunk;
    if ((long long)nchunks != (nblocks + bpc - 1) / bpc) return fail(c, CZ_E_ARG, "chunk count does not match the field");
    if (!d_field) {
        CZ_TRY(grow(c, c->tmp_field, sizeof(float) * (size_t)nx * ny * nz));
        d_field = P<float>(c->tmp_field);
    }
    std::vector<CzField> f(1);
    f[0] = CzField{d_field, nx, ny, nz, p->eps, 0};
    double t[8];
    CZ_TRY(decompress_fields(c, f, nblocks, d_data, d_off, nchunks, p->encoder, p->wtype, p->shuffle, bpc, nullptr,
                             nullptr, 0, (cudaStream_t)stream, d_ref, t));
    // {e_inf, n_inf, e_1, e_2, n_1, n_2, min, max} -> the header's order
    stats[0] = t[0];
    stats[1] = t[1];
    stats[2] = t[2];
    stats[3] = t[4];
    stats[4] = t[3];
    stats[5] = t[5];
    stats[6] = t[6];
    stats[7] = t[7];
    stats[8] = (double)nx * ny * nz;
    return CZ_OK;
}

int cz_res_line(const double *st, long long compressed_bytes, char *buf, int len)
{
    if (!st || !buf || len < 1 || st[8] <= 0) return CZ_E_ARG;
    // Tools/cz2diff.cpp:228-261
    const double n = st[8], e_inf = st[0], n_inf = st[1], e_1 = st[2], n_1 = st[3], e_2 = st[4], n_2 = st[5];
    const double uncompressed = sizeof(float) * n, compressed = (double)compressed_bytes;
    const long double mse = e_2 / n;
    const double psnr = 20 * log10((st[7] - st[6]) / (2 * sqrt(mse)));
    const int w = snprintf(buf, (size_t)len, "RES: %12.2f %.6e %.6e %.6e %.6e %.6e %12.04f %12.04f",
                           uncompressed / compressed, e_inf / n_inf, e_1 / n_1, e_1 / n, sqrt(e_2) / sqrt(n_2),
                           sqrt(e_2) / n, compressed * 8. / n, psnr);
    return w < len ? CZ_OK : CZ_E_SPACE;
}

// After a TMA transpose: the kernel's error flag (a bounded mbarrier wait
// that ran out); waits for the stream.
static int ingest_check(cz_ctx *c, cudaStream_t st)
{
    CZ_TRY(grow_pin(c, 4096));
    int *h = reinterpret_cast<int *>(c->pin);
    CZ_CUDA(c, cudaMemcpyAsync(h, c->ierr.p, 4, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    if (*h != 0) return fail(c, CZ_E_CUDA, "layout transform: a tile copy did not complete");
    return CZ_OK;
}

int cz_field_from_zfastest(cz_ctx *c, const void *d_in, int bytes, int nch, int ch, int nx, int ny, int nz,
                           float *d_field, void *stream)
{
    if (!c || !d_in || !d_field || (bytes != 4 && bytes != 8) || nch < 1 || ch < 0 || ch >= nch || nx < 1 || ny < 1 ||
        nz < 1 || ny > 65535)
        return fail(c, CZ_E_ARG, "bad layout arguments");
    CZ_TRY(set_device(c));
    cudaStream_t st = (cudaStream_t)stream;
    CZ_TRY(grow(c, c->ierr, 64));
    CZ_CUDA(c, cudaMemsetAsync(c->ierr.p, 0, 4, st));
    bool tma = false;
    CZ_CUDA(c, cz_launch_from_zfastest(d_in, bytes, nch, ch, nx, ny, nz, d_field, st, P<int>(c->ierr), &tma));
    return tma ? ingest_check(c, st) : CZ_OK;
}

int cz_field_to_zfastest(cz_ctx *c, const float *d_field, int nx, int ny, int nz, int nch, int ch, float *d_out,
                         void *stream)
{
    if (!c || !d_field || !d_out || nch < 1 || ch < 0 || ch >= nch || nx < 1 || ny < 1 || nz < 1 || ny > 65535)
        return fail(c, CZ_E_ARG, "bad layout arguments");
    CZ_TRY(set_device(c));
    cudaStream_t st = (cudaStream_t)stream;
    CZ_TRY(grow(c, c->ierr, 64));
    CZ_CUDA(c, cudaMemsetAsync(c->ierr.p, 0, 4, st));
    bool tma = false;
    CZ_CUDA(c, cz_launch_to_zfastest(d_field, nx, ny, nz, nch, ch, d_out, st, P<int>(c->ierr), &tma));
    return tma ? ingest_check(c, st) : CZ_OK;
}

int cz_batch_compress(cz_ctx *c, int nfields, const float *const *d_fields, const int *dims, const float *eps,
                      const cz_params *p, void *stream, cz_stream *out)
{
    if (!c || nfields <= 0 || !d_fields || !dims || !eps || !out) return fail(c, CZ_E_ARG, "bad batch arguments");
    CZ_TRY(check_params(c, p));
    CZ_TRY(set_device(c));
    std::vector<CzField> f(nfields);
    long long total = 0;
    for (int i = 0; i < nfields; ++i) {
        CZ_TRY(check_dims(c, dims[3 * i], dims[3 * i + 1], dims[3 * i + 2]));
        if (!d_fields[i]) return fail(c, CZ_E_ARG, "NULL field in batch");
        CZ_TRY(check_align16(c, d_fields[i], "every batch field"));
        f[i] = CzField{d_fields[i], dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], eps[i], total};
        total += (long long)(dims[3 * i] / 32) * (dims[3 * i + 1] / 32) * (dims[3 * i + 2] / 32);
    }
    cz_params q = *p;
    // chunks never straddle fields: one record per chunk in batched mode
    q.blocks_per_chunk = 1;
    cz_stream all;
    CZ_TRY(compress_fields(c, f, total, &q, (cudaStream_t)stream, &all));
    // per-field views into the shared stream (chunk c = block c)
    for (int i = 0; i < nfields; ++i) {
        const long long nb = (long long)(dims[3 * i] / 32) * (dims[3 * i + 1] / 32) * (dims[3 * i + 2] / 32);
        out[i].data = all.data;
        out[i].chunk_offsets = all.chunk_offsets + f[i].block0;
        out[i].nchunks = (int)nb;
        out[i].nblocks = nb;
        out[i].data_bytes = -1;  // per-field sizes: chunk_offsets[nb] - chunk_offsets[0]
        out[i].raw_bytes = -1;
    }
    return CZ_OK;
}

// ------------------------------------------------------------ batch plans
struct cz_plan {
    cz_ctx *c = nullptr;  // private context: its buffers are sized once, so the graph's pointers stay valid
    Job job;
    std::vector<long long> block0;
    std::vector<int> nb;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // autotuner timings (-1: not tuned): the LZ4 stage at 2, 4, 8, 16 chunks
    // per CTA, the wavelet kernel in its two row-prefetch variants
    float lz_ms[4] = {-1.f, -1.f, -1.f, -1.f};
    float enc_ms[2] = {-1.f, -1.f};
};

int cz_plan_destroy(cz_plan *pl)
{
    if (!pl) return CZ_OK;
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->st) cudaStreamDestroy(pl->st);
    if (pl->c) cz_destroy(pl->c);
    delete pl;
    return CZ_OK;
}

int cz_plan_create(cz_ctx *c, int nfields, const float *const *d_fields, const int *dims, const float *eps,
                   const cz_params *p, int tune, cz_plan **out)
{
    if (!c || nfields <= 0 || !d_fields || !dims || !eps || !out) return fail(c, CZ_E_ARG, "bad batch arguments");
    CZ_TRY(check_params(c, p));
    CZ_TRY(set_device(c));
    *out = nullptr;
    std::vector<CzField> f(nfields);
    cz_plan *pl = new cz_plan();
    long long total = 0;
    for (int i = 0; i < nfields; ++i) {
        int rc = check_dims(c, dims[3 * i], dims[3 * i + 1], dims[3 * i + 2]);
        if (rc == CZ_OK && d_fields[i]) rc = check_align16(c, d_fields[i], "every batch field");
        if (rc != CZ_OK || !d_fields[i]) {
            cz_plan_destroy(pl);
            return rc != CZ_OK ? rc : fail(c, CZ_E_ARG, "NULL field in batch");
        }
        f[i] = CzField{d_fields[i], dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], eps[i], total};
        pl->block0.push_back(total);
        pl->nb.push_back((dims[3 * i] / 32) * (dims[3 * i + 1] / 32) * (dims[3 * i + 2] / 32));
        total += pl->nb.back();
    }
    cz_params q = *p;
    q.blocks_per_chunk = 1;  // chunks never straddle fields
    auto bail = [&](int rc, const std::string &msg) {
        if (pl->c && !pl->c->err.empty()) c->err = pl->c->err;
        else c->err = msg;
        cz_plan_destroy(pl);
        return rc;
    };
    int rc = cz_create(c->device, &pl->c);
    if (rc != CZ_OK) return bail(rc, "plan context");
    pl->c->lz_effort = c->lz_effort;
    if (cudaStreamCreateWithFlags(&pl->st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return bail(CZ_E_CUDA, "plan stream");
    }
    if ((rc = prepare(pl->c, f, total, &q, 0, pl->st, pl->job)) != CZ_OK) return bail(rc, "prepare");
    // autotuner, timed on this batch with CUDA events (best of the second
    // and third run of each shape): first the LZ4 stage's CTA width (2, 4,
    // 8 or 16 chunks per CTA) with the wavelet kernel's default variant,
    // then the wavelet kernel's row-prefetch variant with that width. Every
    // shape writes the same bytes.
    cz_stream tmp;
    if (tune) {
        pl->c->timing = true;
        auto time_stage = [&](int stage, float &best_t) -> int {
            float t = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                int r = enqueue(pl->c, pl->job, pl->st, true);
                if (r == CZ_OK) r = finish(pl->c, pl->job, pl->st, &tmp);
                if (r != CZ_OK) return r;
                collect(pl->c);
                if (rep > 0) t = std::min(t, pl->c->stage_ms[stage]);
            }
            best_t = t;
            return CZ_OK;
        };
        if (q.encoder == CZ_ENCODER_LZ4) {
            const int cand[4] = {2, 4, 8, 16};
            int pick = 4;
            float best = 1e30f;
            for (int k = 0; k < 4; ++k) {
                pl->job.lz_warps = cand[k];
                if ((rc = time_stage(1, pl->lz_ms[k])) != CZ_OK) return bail(rc, "tune");
                if (pl->lz_ms[k] < best) {
                    best = pl->lz_ms[k];
                    pick = cand[k];
                }
            }
            pl->job.lz_warps = pick;
        }
        int vpick = 0;
        for (int v = 0; v < 2; ++v) {
            pl->job.enc_variant = v;
            if ((rc = time_stage(0, pl->enc_ms[v])) != CZ_OK) return bail(rc, "tune");
            if (pl->enc_ms[v] < pl->enc_ms[vpick]) vpick = v;
        }
        pl->job.enc_variant = vpick;
        pl->c->timing = false;
    }
    // one graph: memsets, wavelet kernel, chunk setup, scans, LZ4, gather
    if (cudaStreamBeginCapture(pl->st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaGetLastError();
        return bail(CZ_E_CUDA, "stream capture");
    }
    rc = enqueue(pl->c, pl->job, pl->st, false);
    const cudaError_t ec = cudaStreamEndCapture(pl->st, &pl->graph);
    if (rc != CZ_OK || ec != cudaSuccess) {
        cudaGetLastError();
        return bail(rc != CZ_OK ? rc : CZ_E_CUDA, "stream capture");
    }
    if (cudaGraphInstantiate(&pl->exec, pl->graph, 0) != cudaSuccess) {
        cudaGetLastError();
        return bail(CZ_E_CUDA, "graph instantiation");
    }
    *out = pl;
    return CZ_OK;
}

int cz_plan_launch(cz_plan *pl, void *stream)
{
    if (!pl || !pl->exec) return CZ_E_ARG;
    if (cudaGraphLaunch(pl->exec, (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return CZ_E_CUDA;
    }
    return CZ_OK;
}

int cz_plan_result(cz_plan *pl, void *stream, cz_stream *all, cz_stream *per_field)
{
    if (!pl || !all) return CZ_E_ARG;
    CZ_TRY(finish(pl->c, pl->job, (cudaStream_t)stream, all));
    if (per_field)
        for (size_t i = 0; i < pl->nb.size(); ++i) {
            per_field[i].data = all->data;
            per_field[i].chunk_offsets = all->chunk_offsets + pl->block0[i];
            per_field[i].nchunks = pl->nb[i];
            per_field[i].nblocks = pl->nb[i];
            per_field[i].data_bytes = -1;
            per_field[i].raw_bytes = -1;
        }
    return CZ_OK;
}

int cz_plan_info(const cz_plan *pl, int *lz_warps, float *tune_ms)
{
    if (!pl) return CZ_E_ARG;
    if (lz_warps) *lz_warps = pl->job.lz_warps;
    if (tune_ms)
        for (int k = 0; k < 3; ++k) tune_ms[k] = pl->lz_ms[k];
    return CZ_OK;
}

int cz_plan_shape(const cz_plan *pl, int *shape, float *ms)
{
    if (!pl) return CZ_E_ARG;
    if (shape) {
        shape[0] = pl->job.lz_warps;
        shape[1] = pl->job.enc_variant;
    }
    if (ms) {
        for (int k = 0; k < 4; ++k) ms[k] = pl->lz_ms[k];
        for (int v = 0; v < 2; ++v) ms[4 + v] = pl->enc_ms[v];
    }
    return CZ_OK;
}

const char *cz_plan_last_error(const cz_plan *pl) { return pl && pl->c ? pl->c->err.c_str() : ""; }

// ---------------------------------------------------------------- per block
int cz_block_compress(cz_ctx *c, const float *in, float eps, int wtype, int zerobits, int shuffle, uint8_t *out,
                      int *nbytes)
{
    if (!c || !in || !out || !nbytes) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(set_device(c));
    CZ_TRY(grow(c, c->tmp_field, sizeof(float) * kBS3));
    CZ_CUDA(c, cudaMemcpy(c->tmp_field.p, in, sizeof(float) * kBS3, cudaMemcpyHostToDevice));
    cz_params p = {eps, wtype, zerobits, shuffle, CZ_ENCODER_NONE, 1};
    cz_stream s;
    CZ_TRY(cz_field_compress(c, P<float>(c->tmp_field), 32, 32, 32, &p, nullptr, &s));
    int nb = 0;
    CZ_CUDA(c, cudaMemcpy(&nb, s.data, 4, cudaMemcpyDeviceToHost));
    if (nb < kMaskBytes || nb > kMaxRecord) return fail(c, CZ_E_CUDA, "record size out of range");
    CZ_CUDA(c, cudaMemcpy(out, s.data + 4, nb, cudaMemcpyDeviceToHost));
    *nbytes = nb;
    return CZ_OK;
}

int cz_block_decompress(cz_ctx *c, const uint8_t *in, int nbytes, int wtype, int shuffle, float *out)
{
    if (!c || !in || !out) return fail(c, CZ_E_ARG, "NULL argument");
    if (nbytes < kMaskBytes || nbytes > kMaxRecord + 4) return fail(c, CZ_E_CORRUPT, "record size out of range");
    CZ_TRY(set_device(c));
    CZ_TRY(grow(c, c->tmp_field, sizeof(float) * kBS3));
    const size_t need = 16 + (size_t)kSlotBytes;
    CZ_TRY(grow(c, c->tmp_in, need));
    CZ_TRY(grow_pin(c, std::max<size_t>(4096, need)));
    uint8_t *h = reinterpret_cast<uint8_t *>(c->pin);
    long long off[2] = {16, 16 + 4 + (long long)nbytes};
    memcpy(h, off, 16);
    memcpy(h + 16, &nbytes, 4);
    memcpy(h + 20, in, nbytes);
    CZ_CUDA(c, cudaMemcpy(c->tmp_in.p, h, 20 + nbytes, cudaMemcpyHostToDevice));
    cz_params p = {0.f, wtype, 0, shuffle, CZ_ENCODER_NONE, 1};
    // offsets live at the start of tmp_in, the chunk right after them
    CZ_TRY(cz_field_decompress(c, P<uint8_t>(c->tmp_in), P<long long>(c->tmp_in), 1, 32, 32, 32, &p, nullptr,
                               P<float>(c->tmp_field)));
    CZ_CUDA(c, cudaMemcpy(out, c->tmp_field.p, sizeof(float) * kBS3, cudaMemcpyDeviceToHost));
    return CZ_OK;
}

// ---------------------------------------------------------------- LZ4
int cz_lz4_bound(int isize) { return isize < 0 ? 0 : isize + isize / 255 + 16; }

int cz_lz4_compress(cz_ctx *c, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out)
{
    if (!c || (!src && isize) || !dst || !out || isize < 0) return fail(c, CZ_E_ARG, "bad LZ4 arguments");
    CZ_TRY(set_device(c));
    const long long bound = lz4_bound_ll(isize);
    const size_t in_bytes = (size_t)isize + 64;
    CZ_TRY(grow(c, c->tmp_in, in_bytes + 64 + (size_t)bound + 64));
    CZ_TRY(grow_pin(c, 4096));
    uint8_t *d = P<uint8_t>(c->tmp_in);
    const size_t meta = in_bytes + 64 - (in_bytes + 64) % 16;  // 16-aligned area after the input
    uint8_t *dout = d + meta + 64;
    long long *h = reinterpret_cast<long long *>(c->pin);
    h[0] = 0;                 // in_off
    h[1] = 0;                 // out_off
    reinterpret_cast<int *>(h + 2)[0] = isize;
    if (isize) CZ_CUDA(c, cudaMemcpy(d, src, isize, cudaMemcpyHostToDevice));
    CZ_CUDA(c, cudaMemcpy(d + meta, h, 24, cudaMemcpyHostToDevice));
    long long *doff = reinterpret_cast<long long *>(d + meta);
    int *dlen = reinterpret_cast<int *>(d + meta + 16);
    int *dout_len = reinterpret_cast<int *>(d + meta + 20);
    CZ_CUDA(c, cz_launch_lz4_encode(d, doff, dlen, 1, dout, doff + 1, dout_len, 0, 4, 1, nullptr, nullptr,
                                    c->lz_effort));
    int n = 0;
    CZ_CUDA(c, cudaMemcpy(&n, dout_len, 4, cudaMemcpyDeviceToHost));
    if (n < 0) return fail(c, CZ_E_CUDA, "LZ4 encoder output exceeded its bound");
    if (n > cap) return fail(c, CZ_E_SPACE, "LZ4 output buffer too small");
    CZ_CUDA(c, cudaMemcpy(dst, dout, n, cudaMemcpyDeviceToHost));
    *out = n;
    return CZ_OK;
}

int cz_zlib_bound(int isize) { return isize < 0 ? 0 : (int)zlib_bound_ll(isize); }

int cz_zlib_compress(cz_ctx *c, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out)
{
    if (!c || (!src && isize) || !dst || !out || isize < 0 || isize > (1 << 24) - 64)
        return fail(c, CZ_E_ARG, "bad zlib arguments");
    CZ_TRY(set_device(c));
    const size_t in_bytes = ((size_t)isize + 64 + 15) / 16 * 16;
    const size_t seq_bytes = ((size_t)seq_bound_ll(isize) + 15) / 16 * 16;
    const size_t zbytes = ((size_t)zlib_bound_ll(isize) + 16 + 15) / 16 * 16;
    CZ_TRY(grow(c, c->tmp_in, in_bytes + 64 + seq_bytes + zbytes));
    CZ_TRY(grow_pin(c, 4096));
    uint8_t *d = P<uint8_t>(c->tmp_in);
    uint8_t *meta = d + in_bytes;  // in_off, seq_off, zoff (8 each), in_len, seq_len, zlen (4 each)
    uint8_t *dseq = meta + 64, *dz = dseq + seq_bytes;
    long long *h = reinterpret_cast<long long *>(c->pin);
    h[0] = 0;
    h[1] = 0;
    h[2] = 0;
    reinterpret_cast<int *>(h + 3)[0] = isize;
    if (isize) CZ_CUDA(c, cudaMemcpy(d, src, isize, cudaMemcpyHostToDevice));
    CZ_CUDA(c, cudaMemcpy(meta, h, 32, cudaMemcpyHostToDevice));
    long long *doff = reinterpret_cast<long long *>(meta);
    int *dlen = reinterpret_cast<int *>(meta + 24);
    CZ_CUDA(c, cz_launch_lz77_parse(d, doff, dlen, 1, dseq, doff + 1, dlen + 1, 0, 1, nullptr, c->lz_effort));
    CZ_CUDA(c, cz_launch_deflate(d, doff, dlen, dseq, doff + 1, dlen + 1, 1, 0, dz, (long long)zbytes, doff + 2,
                                 dlen + 2, 1, nullptr));
    int n = 0;
    CZ_CUDA(c, cudaMemcpy(&n, dlen + 2, 4, cudaMemcpyDeviceToHost));
    if (n < 0) return fail(c, CZ_E_CUDA, "zlib encoder failed");
    if (n > cap) return fail(c, CZ_E_SPACE, "zlib output buffer too small");
    CZ_CUDA(c, cudaMemcpy(dst, dz, n, cudaMemcpyDeviceToHost));
    *out = n;
    return CZ_OK;
}

int cz_lz4_decompress(cz_ctx *c, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out)
{
    if (!c || (!src && isize) || !dst || !out || isize < 0 || cap < 0) return fail(c, CZ_E_ARG, "bad LZ4 arguments");
    CZ_TRY(set_device(c));
    const size_t in_bytes = ((size_t)isize + 64 + 15) / 16 * 16;
    CZ_TRY(grow(c, c->tmp_in, in_bytes + 64 + (size_t)cap + 64));
    CZ_TRY(grow_pin(c, 4096));
    uint8_t *d = P<uint8_t>(c->tmp_in);
    uint8_t *meta = d + in_bytes;
    uint8_t *dout = meta + 64;
    long long *h = reinterpret_cast<long long *>(c->pin);
    h[0] = 0;
    h[1] = 0;
    reinterpret_cast<int *>(h + 2)[0] = isize;
    reinterpret_cast<int *>(h + 2)[1] = cap;
    if (isize) CZ_CUDA(c, cudaMemcpy(d, src, isize, cudaMemcpyHostToDevice));
    CZ_CUDA(c, cudaMemcpy(meta, h, 24, cudaMemcpyHostToDevice));
    long long *doff = reinterpret_cast<long long *>(meta);
    int *dlen = reinterpret_cast<int *>(meta + 16);
    int *dcap = reinterpret_cast<int *>(meta + 20);
    int *dres = reinterpret_cast<int *>(meta + 24);
    CZ_CUDA(c, cz_launch_lz4_decode(d, doff, dlen, 1, dout, doff + 1, dcap, dres, 1, nullptr));
    int n = 0;
    CZ_CUDA(c, cudaMemcpy(&n, dres, 4, cudaMemcpyDeviceToHost));
    *out = n;
    if (n < 0) return fail(c, CZ_E_CORRUPT, "malformed LZ4 input");
    if (n) CZ_CUDA(c, cudaMemcpy(dst, dout, n, cudaMemcpyDeviceToHost));
    return CZ_OK;
}

int cz_zlib_decompress(cz_ctx *c, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out)
{
    if (!c || (!src && isize) || !dst || !out || isize < 0 || cap < 0) return fail(c, CZ_E_ARG, "bad zlib arguments");
    CZ_TRY(set_device(c));
    const size_t in_bytes = ((size_t)isize + 64 + 15) / 16 * 16;
    CZ_TRY(grow(c, c->tmp_in, in_bytes + 64 + (size_t)cap + 64));
    CZ_TRY(grow_pin(c, 4096));
    uint8_t *d = P<uint8_t>(c->tmp_in);
    uint8_t *meta = d + in_bytes;
    uint8_t *dout = meta + 64;
    long long *h = reinterpret_cast<long long *>(c->pin);
    h[0] = 0;
    h[1] = 0;
    reinterpret_cast<int *>(h + 2)[0] = isize;
    reinterpret_cast<int *>(h + 2)[1] = cap;
    if (isize) CZ_CUDA(c, cudaMemcpy(d, src, isize, cudaMemcpyHostToDevice));
    CZ_CUDA(c, cudaMemcpy(meta, h, 24, cudaMemcpyHostToDevice));
    long long *doff = reinterpret_cast<long long *>(meta);
    int *dlen = reinterpret_cast<int *>(meta + 16);
    int *dcap = reinterpret_cast<int *>(meta + 20);
    int *dres = reinterpret_cast<int *>(meta + 24);
    CZ_CUDA(c, cz_launch_inflate(d, doff, dlen, 1, dout, doff + 1, dcap, dres, 1, nullptr));
    int n = 0;
    CZ_CUDA(c, cudaMemcpy(&n, dres, 4, cudaMemcpyDeviceToHost));
    *out = n;
    if (n < 0) return fail(c, CZ_E_CORRUPT, "malformed zlib input");
    if (n) CZ_CUDA(c, cudaMemcpy(dst, dout, n, cudaMemcpyDeviceToHost));
    return CZ_OK;
}

// ---------------------------------------------------------------- .cz images
long long cz_file_bytes(cz_ctx *c, const cz_stream *s, int nx, int ny, int nz, const cz_params *p)
{
    if (!s || !p || check_dims(c, nx, ny, nz) != CZ_OK) return -1;
    const std::string hdr = czf::header_text(nx / 32, ny / 32, nz / 32, p->eps, p->wtype, p->encoder);
    return czf::image_bytes(s->data_bytes, s->nchunks, s->nblocks, hdr);
}

int cz_file_image(cz_ctx *c, const cz_stream *s, int nx, int ny, int nz, const cz_params *p, uint8_t *out,
                  long long cap, long long *written)
{
    if (!c || !s || !p || !out || !written) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(set_device(c));
    const int bx = nx / 32, by = ny / 32, bz = nz / 32;
    const long long nblocks = (long long)bx * by * bz;
    if (s->nblocks != nblocks) return fail(c, CZ_E_ARG, "stream does not match the field extents");
    const std::string hdr = czf::header_text(bx, by, bz, p->eps, p->wtype, p->encoder);
    const long long need = czf::image_bytes(s->data_bytes, s->nchunks, nblocks, hdr);
    if (need > cap) return fail(c, CZ_E_SPACE, "image buffer too small");
    std::vector<long long> off(s->nchunks + 1);
    CZ_CUDA(c, cudaMemcpy(off.data(), s->chunk_offsets, sizeof(long long) * (s->nchunks + 1), cudaMemcpyDeviceToHost));
    const long long base = off[0];
    for (auto &o : off) o -= base;
    // payloads land directly in the caller's buffer behind the mini header
    uint8_t *payload = out + czf::mini_header_bytes();
    CZ_CUDA(c, cudaMemcpy(payload, s->data + base, (size_t)off[s->nchunks], cudaMemcpyDeviceToHost));
    const int bpc = std::max(1, (int)((nblocks + s->nchunks - 1) / s->nchunks));
    std::vector<int> bc(nblocks), bs(nblocks);
    for (long long g = 0; g < nblocks; ++g) {
        bc[g] = (int)(g / bpc);
        bs[g] = (int)(g % bpc);
    }
    *written = czf::write_image(out, payload, off[s->nchunks], off.data(), s->nchunks, bc.data(), bs.data(), bx, by,
                                bz, hdr);
    return CZ_OK;
}

namespace {

constexpr int kSlabs = 16;

// Streams of the pipelined path: the wavelet kernels on the highest
// priority (their CTAs are scheduled before pending LZ4 CTAs), the LZ4
// stages on the lowest.
int pipeline_streams(cz_ctx *c)
{
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
        cudaGetLastError();
        least = greatest = 0;
    }
    auto mk = [&](cudaStream_t &st, int prio) {
        if (!st && cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio) != cudaSuccess) {
            cudaGetLastError();
            return fail(c, CZ_E_CUDA, "stream creation failed");
        }
        return CZ_OK;
    };
    CZ_TRY(mk(c->s_copy, 0));
    CZ_TRY(mk(c->s_gather, 0));
    CZ_TRY(mk(c->s_comp, greatest));
    while ((int)c->s_lz.size() < kSlabs) {
        cudaStream_t st = nullptr;
        CZ_TRY(mk(st, least));
        c->s_lz.push_back(st);
    }
    for (auto *v : {&c->ev_h2d, &c->ev_enc, &c->ev_lz})
        while ((int)v->size() < kSlabs) {
            cudaEvent_t e;
            CZ_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            v->push_back(e);
        }
    if (!c->ev_join) CZ_CUDA(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    return CZ_OK;
}

}  // namespace

// Host field in, .cz image in host memory out, pipelined over z-slabs of
// whole block layers: the slabs' host-to-device copies run on a copy
// stream; the wavelet kernel of slab i waits only for slab i's copy; slab
// i's LZ4 stage runs on its own stream (a chunk's LZ4 is one warp's serial
// work, so slabs overlap); the gather stream keeps the running prefix sum
// of chunk sizes and writes each slab's chunks straight into the caller's
// image when it is device-accessible host memory (else into the device
// stream buffer, copied once at the end). The header, metadata and LUT are
// written on the host after the last slab.
int cz_compress_to_image(cz_ctx *c, const float *h_field, int nx, int ny, int nz, const cz_params *p, void *stream,
                         uint8_t *out, long long cap, long long *written)
{
    if (!c || !h_field || !out || !written) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(check_params(c, p));
    CZ_TRY(check_dims(c, nx, ny, nz));
    CZ_TRY(set_device(c));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(float) * (size_t)nx * ny * nz;
    CZ_TRY(grow(c, c->tmp_field, bytes));
    if (p->blocks_per_chunk != 1 || p->encoder == CZ_ENCODER_ZLIB) {  // whole-field path
        CZ_CUDA(c, cudaMemcpyAsync(c->tmp_field.p, h_field, bytes, cudaMemcpyHostToDevice, st));
        cz_stream s;
        CZ_TRY(cz_field_compress(c, P<float>(c->tmp_field), nx, ny, nz, p, stream, &s));
        return cz_file_image(c, &s, nx, ny, nz, p, out, cap, written);
    }
    const int bx = nx / 32, by = ny / 32, bz = nz / 32;
    const long long layer = (long long)bx * by;  // blocks (and chunks) per block layer
    const long long nblocks = layer * bz;
    const int nslab = std::min(bz, kSlabs);
    const bool lz4 = p->encoder == CZ_ENCODER_LZ4;
    CZ_TRY(pipeline_streams(c));
    // buffers for the whole field (the slabs index into them)
    std::vector<CzField> slabs(nslab);
    std::vector<long long> first(nslab + 1);
    for (int i = 0; i <= nslab; ++i) first[i] = layer * (long long)((long long)bz * i / nslab);
    for (int i = 0; i < nslab; ++i) {
        const long long z0 = 32 * (first[i] / layer), depth = 32 * ((first[i + 1] - first[i]) / layer);
        slabs[i] = CzField{P<float>(c->tmp_field) + z0 * ny * nx, nx, ny, (int)depth, p->eps, 0};
    }
    Job job;
    CZ_TRY(prepare(c, slabs, nblocks, p, 0, st, job));
    CZ_TRY(grow(c, c->queue, 8 * kSlabs + 64));
    // the payload goes straight to the image when the device can write it
    const std::string hdr = czf::header_text(bx, by, bz, p->eps, p->wtype, p->encoder);
    const long long mini = czf::mini_header_bytes();
    const long long bound = (long long)job.nchunks * (lz4 ? job.lz_slot : kSlotBytes);
    uint8_t *direct = nullptr;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        cap >= czf::image_bytes(bound, job.nchunks, nblocks, hdr))
        direct = static_cast<uint8_t *>(pa.devicePointer) + mini;
    cudaGetLastError();
    uint8_t *dst = direct ? direct : P<uint8_t>(c->out_data);
    CZ_CUDA(c, cudaMemsetAsync(c->queue.p, 0, 8 * kSlabs, st));
    CZ_CUDA(c, cudaMemsetAsync(c->flag.p, 0, 64, st));
    CZ_CUDA(c, cudaMemsetAsync(c->out_off.p, 0, 8, st));
    CZ_CUDA(c, cudaEventRecord(c->ev_join, st));
    CZ_CUDA(c, cudaStreamWaitEvent(c->s_gather, c->ev_join, 0));
    CZ_CUDA(c, cudaStreamWaitEvent(c->s_copy, c->ev_join, 0));
    CZ_CUDA(c, cudaStreamWaitEvent(c->s_comp, c->ev_join, 0));
    cudaStream_t cs = c->s_comp;
    for (int i = 0; i < nslab; ++i) {
        const size_t off = (size_t)(first[i] / layer) * 32 * ny * nx, n = (size_t)(first[i + 1] - first[i]) / layer * 32 * ny * nx;
        CZ_CUDA(c, cudaMemcpyAsync(P<float>(c->tmp_field) + off, h_field + off, n * sizeof(float),
                                   cudaMemcpyHostToDevice, c->s_copy));
        CZ_CUDA(c, cudaEventRecord(c->ev_h2d[i], c->s_copy));
    }
    unsigned long long *queues = P<unsigned long long>(c->queue);
    for (int i = 0; i < nslab; ++i) {
        const long long f0 = first[i];
        const int n = (int)(first[i + 1] - f0);
        uint8_t *stage = P<uint8_t>(c->stage) + f0 * kSlotBytes;
        CZ_CUDA(c, cudaStreamWaitEvent(cs, c->ev_h2d[i], 0));
        CZ_CUDA(c, cz_launch_encode(p->wtype, P<CzField>(c->fields) + i, 1, n, p->zerobits, p->shuffle ? 1 : 0, stage,
                                    P<int>(c->rec_bytes) + f0, queues + i, std::min(n, c->sms), cs));
        CZ_CUDA(c, cz_launch_chunk_setup(1, n, n, P<int>(c->rec_bytes) + f0, P<long long>(c->in_off) + f0,
                                         P<int>(c->in_len) + f0, nullptr, P<long long>(c->lz_off) + f0, job.lz_slot,
                                         cs));
        CZ_CUDA(c, cudaEventRecord(c->ev_enc[i], cs));
        const uint8_t *src = stage;
        const long long *src_off = P<long long>(c->in_off) + f0;
        const int *len = P<int>(c->in_len) + f0;
        cudaEvent_t ready = c->ev_enc[i];
        if (lz4) {
            cudaStream_t ls = c->s_lz[i];
            CZ_CUDA(c, cudaStreamWaitEvent(ls, c->ev_enc[i], 0));
            uint8_t *lzo = P<uint8_t>(c->lz_out) + f0 * job.lz_slot;
            // whole-SM CTAs (16 chunks each): LZ4 and the wavelet kernel of
            // the next slabs then share the GPU SM by SM
            const int lzgrid = std::max(1, std::min((n + 15) / 16, c->sms));
            CZ_CUDA(c, cz_launch_lz4_encode(stage, src_off, len, n, lzo, P<long long>(c->lz_off) + f0,
                                            P<int>(c->lz_len) + f0, p->shuffle ? 1 : 0, 16, lzgrid, ls,
                                            P<int4>(c->lz_hole) + f0, c->lz_effort));
            CZ_CUDA(c, cz_launch_neg_reduce(P<int>(c->lz_len) + f0, n, P<int>(c->flag), ls));
            CZ_CUDA(c, cudaEventRecord(c->ev_lz[i], ls));
            src = lzo;
            src_off = P<long long>(c->lz_off) + f0;
            len = P<int>(c->lz_len) + f0;
            ready = c->ev_lz[i];
        }
        CZ_CUDA(c, cudaStreamWaitEvent(c->s_gather, ready, 0));
        CZ_CUDA(c, cz_launch_scan_from(len, n, P<long long>(c->out_off) + f0, c->s_gather));
        CZ_CUDA(c, cz_launch_gather(src, src_off, len, n, dst, P<long long>(c->out_off) + f0, c->s_gather,
                                    lz4 ? P<int4>(c->lz_hole) + f0 : nullptr, stage, P<long long>(c->in_off) + f0));
    }
    CZ_CUDA(c, cudaEventRecord(c->ev_join, c->s_gather));
    CZ_CUDA(c, cudaStreamWaitEvent(st, c->ev_join, 0));
    // sizes and offsets back, then the host-side tail
    std::vector<long long> off(job.nchunks + 1);
    int flag = 0;
    CZ_CUDA(c, cudaMemcpyAsync(off.data(), c->out_off.p, sizeof(long long) * (job.nchunks + 1), cudaMemcpyDeviceToHost,
                               st));
    CZ_CUDA(c, cudaMemcpyAsync(&flag, c->flag.p, 4, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    if (flag != 0) return fail(c, CZ_E_CUDA, "LZ4 encoder output exceeded its bound");
    const long long payload = off[job.nchunks];
    const long long need = czf::image_bytes(payload, job.nchunks, nblocks, hdr);
    if (need > cap) return fail(c, CZ_E_SPACE, "image buffer too small");
    if (!direct) CZ_CUDA(c, cudaMemcpy(out + mini, dst, (size_t)payload, cudaMemcpyDeviceToHost));
    std::vector<int> bc(nblocks), bsub(nblocks, 0);
    for (long long g = 0; g < nblocks; ++g) bc[g] = (int)g;
    *written = czf::write_image(out, out + mini, payload, off.data(), job.nchunks, bc.data(), bsub.data(), bx, by, bz,
                                hdr);
    c->nblocks = nblocks;
    c->nchunks = job.nchunks;
    c->bpc = 1;
    return CZ_OK;
}

// ---------------------------------------------------- several ranks, one file
long long cz_mini_bytes(void) { return czf::mini_header_bytes(); }

int cz_mini_write(long long header_offset, uint8_t *out, long long cap)
{
    if (!out || cap < czf::mini_header_bytes() || header_offset < czf::mini_header_bytes()) return CZ_E_ARG;
    czf::write_mini(out, header_offset);
    return CZ_OK;
}

long long cz_part_bytes(long long payload_bytes, int nchunks)
{
    if (payload_bytes < 0 || nchunks < 0) return -1;
    return payload_bytes + 8LL * nchunks;
}

int cz_part_write(const uint8_t *payload, const long long *chunk_offsets, int nchunks, uint8_t *out, long long cap,
                  long long *written)
{
    if (!chunk_offsets || !out || !written || nchunks < 1) return CZ_E_ARG;
    if (chunk_offsets[0] != 0) return CZ_E_ARG;
    for (int c = 0; c < nchunks; ++c)
        if (chunk_offsets[c + 1] < chunk_offsets[c]) return CZ_E_ARG;
    const long long bytes = chunk_offsets[nchunks];
    if (bytes > 0 && !payload) return CZ_E_ARG;
    if (cz_part_bytes(bytes, nchunks) > cap) return CZ_E_SPACE;
    *written = czf::write_part(out, payload, bytes, chunk_offsets, nchunks);
    return CZ_OK;
}

int cz_stream_part(cz_ctx *c, const cz_stream *s, uint8_t *out, long long cap, long long *written)
{
    if (!c || !s || !out || !written) return fail(c, CZ_E_ARG, "NULL argument");
    CZ_TRY(set_device(c));
    std::vector<long long> off(s->nchunks + 1);
    CZ_CUDA(c, cudaMemcpy(off.data(), s->chunk_offsets, sizeof(long long) * (s->nchunks + 1), cudaMemcpyDeviceToHost));
    const long long base = off[0];
    for (auto &o : off) o -= base;
    if (cz_part_bytes(off[s->nchunks], s->nchunks) > cap) return fail(c, CZ_E_SPACE, "part buffer too small");
    CZ_CUDA(c, cudaMemcpy(out, s->data + base, (size_t)off[s->nchunks], cudaMemcpyDeviceToHost));
    *written = czf::write_part(out, out, off[s->nchunks], off.data(), s->nchunks);
    return CZ_OK;
}

long long cz_tail_bytes(int bx, int by, int bz, int nranks, const cz_params *p)
{
    if (!p || bx < 1 || by < 1 || bz < 1 || nranks < 1 || bz % nranks) return -1;
    const std::string hdr = czf::header_text_sub(bx, by, bz, bx, by, bz / nranks, p->eps, p->wtype, p->encoder);
    return czf::tail_bytes((long long)bx * by * bz, nranks, hdr);
}

int cz_tail_write(int bx, int by, int bz, int nranks, const long long *part_bytes, const int *part_chunks,
                  const cz_params *p, uint8_t *out, long long cap, long long *written)
{
    if (!p || !part_bytes || !part_chunks || !out || !written) return CZ_E_ARG;
    if (bx < 1 || by < 1 || bz < 1 || nranks < 1 || bz % nranks || p->blocks_per_chunk < 1) return CZ_E_ARG;
    const long long bps = (long long)bx * by * (bz / nranks);
    const long long nch = (bps + p->blocks_per_chunk - 1) / p->blocks_per_chunk;
    for (int r = 0; r < nranks; ++r)
        if (part_chunks[r] != nch || part_bytes[r] < 8LL * nch) return CZ_E_ARG;
    const std::string hdr = czf::header_text_sub(bx, by, bz, bx, by, bz / nranks, p->eps, p->wtype, p->encoder);
    if (czf::tail_bytes((long long)bx * by * bz, nranks, hdr) > cap) return CZ_E_SPACE;
    *written = czf::write_tail(out, hdr, bx, by, bz, nranks, p->blocks_per_chunk, part_bytes, part_chunks);
    return CZ_OK;
}

int cz_image_info(const uint8_t *img, long long size, int *dims, int *encoder)
{
    if (!img || !dims) return CZ_E_ARG;
    czf::Parsed ps;
    std::string err;
    if (czf::parse_image(img, size, ps, err) != 0) return CZ_E_CORRUPT;
    dims[0] = ps.bx * 32;
    dims[1] = ps.by * 32;
    dims[2] = ps.bz * 32;
    if (encoder) *encoder = ps.encoder;
    return CZ_OK;
}

int cz_decompress_image(cz_ctx *c, const uint8_t *img, long long size, int wtype, int shuffle, void *stream,
                        float *h_field, long long field_cap)
{
    if (!c || !img || !h_field) return fail(c, CZ_E_ARG, "NULL argument");
    czf::Parsed ps;
    std::string err;
    if (czf::parse_image(img, size, ps, err) != 0) return fail(c, CZ_E_CORRUPT, err);
    if (ps.wavelets != czf::wavelet_name(wtype))
        return fail(c, CZ_E_ARG, "file wavelets " + ps.wavelets + " do not match wtype " + std::to_string(wtype));
    if (ps.encoder != CZ_ENCODER_NONE && ps.encoder != CZ_ENCODER_LZ4 && ps.encoder != CZ_ENCODER_ZLIB)
        return fail(c, CZ_E_ARG, "unsupported encoder in file");
    const int nx = ps.bx * 32, ny = ps.by * 32, nz = ps.bz * 32;
    const long long nelem = (long long)nx * ny * nz;
    if (field_cap < nelem) return fail(c, CZ_E_SPACE, "output field too small");
    CZ_TRY(set_device(c));
    cudaStream_t st = (cudaStream_t)stream;
    const int nchunks = (int)ps.chunk_start.size();
    const long long nblocks = (long long)ps.bx * ps.by * ps.bz;
    // payloads back to back on the device with a compact offset table;
    // files from several ranks carry each rank's LUT between their chunks,
    // those chunks are compacted on the host first
    bool contiguous = true;
    long long total = 0;
    for (int i = 0; i < nchunks; ++i) {
        if (i + 1 < nchunks && ps.chunk_start[i] + ps.chunk_size[i] != ps.chunk_start[i + 1]) contiguous = false;
        total += ps.chunk_size[i];
    }
    std::vector<long long> off(nchunks + 1);
    long long acc = 0;  // 64-bit: the payload of a file may pass 2 GiB
    for (int i = 0; i < nchunks; ++i) {
        off[i] = contiguous ? ps.chunk_start[i] - ps.chunk_start[0] : acc;
        acc += ps.chunk_size[i];
    }
    off[nchunks] = total;
    for (int i = 0; i < nchunks; ++i)
        if (ps.encoder == CZ_ENCODER_NONE && (off[i] % 4) != 0)
            return fail(c, CZ_E_CORRUPT, "raw chunk payloads are not 4-byte aligned");
    const size_t data_pad = ((size_t)total + 255) / 256 * 256;
    CZ_TRY(grow(c, c->tmp_in, data_pad + sizeof(long long) * (nchunks + 1)));
    CZ_TRY(grow(c, c->tmp_field, sizeof(float) * (size_t)nelem));
    uint8_t *d = P<uint8_t>(c->tmp_in);
    long long *doff = reinterpret_cast<long long *>(d + data_pad);
    if (contiguous) {
        CZ_CUDA(c, cudaMemcpyAsync(d, img + ps.chunk_start[0], (size_t)total, cudaMemcpyHostToDevice, st));
    } else {
        std::vector<uint8_t> packed((size_t)total);
        for (int i = 0; i < nchunks; ++i) memcpy(&packed[off[i]], img + ps.chunk_start[i], ps.chunk_size[i]);
        // on the call's stream: the decode kernels below run there; the
        // synchronisation that follows keeps `packed` alive until the copy ends
        CZ_CUDA(c, cudaMemcpyAsync(d, packed.data(), (size_t)total, cudaMemcpyHostToDevice, st));
    }
    CZ_CUDA(c, cudaMemcpyAsync(doff, off.data(), sizeof(long long) * (nchunks + 1), cudaMemcpyHostToDevice, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    std::vector<CzField> f(1);
    f[0] = CzField{P<float>(c->tmp_field), nx, ny, nz, 0.f, 0};
    CZ_TRY(decompress_fields(c, f, nblocks, d, doff, nchunks, ps.encoder, wtype, shuffle, 1, ps.block_chunk.data(),
                             ps.block_subid.data(), std::max(1, ps.max_subid), st));
    CZ_CUDA(c, cudaMemcpyAsync(h_field, c->tmp_field.p, sizeof(float) * (size_t)nelem, cudaMemcpyDeviceToHost, st));
    CZ_CUDA(c, cudaStreamSynchronize(st));
    return CZ_OK;
}

}  // extern "C"
