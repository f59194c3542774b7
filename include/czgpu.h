/*
 * czgpu.h -- C-ABI of the GB300 wavelet compression path (libczgpu.so).
 *
 * Drop-in for the per-block codec and lossless stage of CubismZ
 * (fab4100/CubismZ). Plain C types only; every entry point returns an int
 * status (CZ_OK or a negative CZ_E* code) and never aborts. Device pointers
 * are CUDA global memory of the context's device; `stream` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).
 *
 * Reference interfaces replaced (paths within the reference project):
 *   WaveletCompressorGeneric<32,float>::compress / decompress
 *       Compressor/source/WaveletCompressor.h:61-71, WaveletCompressor.cpp:152-259
 *   deflate_inplace (LZ4 branch) / zdecompress
 *       Compressor/source/CompressionEncoders.h:45-46, 113-247, 48-88
 *   LZ4_compress / LZ4_uncompress_unknownOutputSize
 *       ThirdParty/lz4/lz4.h:53,112 (lz4.c:695-700, 802-905)
 *   the writer's block loop and .cz layout
 *       Compressor/source/SerializerIO_WaveletCompression_MPI_Simple.h:187-345, 347-466, 489-644
 *   the reader's load_file / load_block2
 *       Compressor/source/Reader_WaveletCompression.h:255-560, 635-754
 */
#ifndef CZGPU_H
#define CZGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CZ_OK 0
#define CZ_E_ARG -1      /* invalid argument (sizes, pointers, parameters) */
#define CZ_E_CUDA -2     /* a CUDA call failed */
#define CZ_E_CORRUPT -3  /* malformed record, LZ4 stream or .cz file */
#define CZ_E_SPACE -4    /* caller buffer too small */
#define CZ_E_NOMEM -5    /* device or host allocation failed */

#define CZ_BLOCKSIZE 32
#define CZ_BLOCK_ELEMS 32768
#define CZ_MASK_BYTES 4096
#define CZ_MAX_RECORD (4096 + 4 * 32768) /* WaveletCompressor.h:40-45 */

#define CZ_ENCODER_NONE 0 /* "Encoder: none"  (CompressionEncoders.h:240-246) */
#define CZ_ENCODER_LZ4 1  /* "Encoder: lz4"   (CompressionEncoders.h:192-238) */
#define CZ_ENCODER_ZLIB 2 /* "Encoder: zlib"  (CompressionEncoders.h:116-190) */

typedef struct cz_ctx cz_ctx;

/* Codec parameters: the reference's compile-time switches as run-time values.
 *   eps        absolute threshold, |c| > eps is kept (FullWaveletTransform.h:84)
 *   wtype      1 interp 4th order, 2 lifted interp, 3 average-interp 3rd order
 *              (any other value behaves as 3, WaveletsOnInterval.h:154)
 *   zerobits   0 or n: clear the n low bits of every survivor (-D_ZEROBITS_=n)
 *   shuffle    0/1: byte-plane shuffle of the survivors (-D_USE_SHUFFLE3_)
 *   encoder    CZ_ENCODER_NONE, CZ_ENCODER_LZ4, or CZ_ENCODER_ZLIB
 *   blocks_per_chunk  records per lossless chunk (1 is the default) */
typedef struct {
    float eps;
    int wtype;
    int zerobits;
    int shuffle;
    int encoder;
    int blocks_per_chunk;
} cz_params;

/* Compressed field held in device memory owned by the context (valid until
 * the next call on the context). data: chunk payloads back to back;
 * chunk_offsets[nchunks+1]: offsets into data (device); nblocks: records in
 * the stream, blocks_per_chunk of them per chunk in block order; raw_bytes:
 * total record bytes before the lossless stage. */
typedef struct {
    const uint8_t *data;
    long long data_bytes;
    const long long *chunk_offsets; /* device */
    int nchunks;
    long long nblocks;
    long long raw_bytes;
} cz_stream;

/* ---- context ---------------------------------------------------------- */
/* New context on `device` (scratch buffers are allocated on first use and
 * grown as needed). Calls on one context must not overlap: use one context
 * per host thread, as the reference uses one compressor object per OpenMP
 * thread; contexts are independent of each other. A cz_stream points into
 * its context's buffers and stays valid until the next call on it. */
int cz_create(int device, cz_ctx **out);
int cz_destroy(cz_ctx *ctx);
/* Last error text of the context (never NULL). */
const char *cz_last_error(cz_ctx *ctx);

/* Per-stage device timing (CUDA events on the call's stream), the
 * counterpart of the writer's fwt/encoding timers
 * (SerializerIO_WaveletCompression_MPI_Simple.h:201-203, 325, 341-343).
 * After cz_set_timing(ctx, 1), every field call records its stages;
 * cz_stage_times writes up to n durations in milliseconds:
 *   compress:   [0] codec kernel, [1] lossless stage, [2] stream assembly
 *   decompress: [0] lossless stage, [1] record location, [2] codec kernel
 * and returns how many were written. */
int cz_set_timing(cz_ctx *ctx, int on);
int cz_stage_times(cz_ctx *ctx, float *ms, int n);

/* Parse effort of the GPU LZ4 encoder (and of the LZ77 parse under the zlib
 * stage) for the context's later calls; plans keep the effort they were
 * created with. Any level yields streams that the reference decoder reads
 * (lz4.c:802-905); higher levels find more matches and take longer:
 *   0  the lane-parallel greedy parse alone (fastest)
 *   1  (default) also extends matches backwards over equal bytes, as
 *      lz4.c's "catch up" does (lz4.c:586-587), and keeps the part of a
 *      match that the match of a lower lane overlaps
 *   2  also takes repeats at distance 1-3 that the hash table misses, and
 *      starts each lane's walk 8 positions early
 * CZ_E_ARG for other values. No counterpart in the reference, whose LZ4 has
 * one level. */
int cz_set_lz4_effort(cz_ctx *ctx, int effort);

/* ---- per-block drop-in (host buffers) --------------------------------- */
/* WaveletCompressor::compress of one 32^3 block in[z][y][x]: writes the
 * record [4096-byte mask][survivors] to out (capacity CZ_MAX_RECORD) and its
 * size to *nbytes. Replaces WaveletCompressor.cpp:152-182. */
int cz_block_compress(cz_ctx *ctx, const float *in, float eps, int wtype, int zerobits, int shuffle, uint8_t *out,
                      int *nbytes);
/* WaveletCompressor::decompress of one record into out[z][y][x].
 * Replaces WaveletCompressor.cpp:231-259 (+ copy_to, WaveletCompressor.h:66-82). */
int cz_block_decompress(cz_ctx *ctx, const uint8_t *in, int nbytes, int wtype, int shuffle, float *out);

/* ---- LZ4 pair (host buffers) ------------------------------------------ */
/* Worst-case output size, LZ4_compressBound (lz4.h:81-82). */
int cz_lz4_bound(int isize);
/* Compress src[0..isize) into dst (capacity cap >= cz_lz4_bound(isize));
 * *out = compressed size. Replaces LZ4_compress (lz4.c:695-700). */
int cz_lz4_compress(cz_ctx *ctx, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out);
/* Decode with the acceptance rules of LZ4_uncompress_unknownOutputSize
 * (lz4.c:802-905); *out = decoded size. Malformed input -> CZ_E_CORRUPT. */
int cz_lz4_decompress(cz_ctx *ctx, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out);
/* Worst-case zlib stream size of cz_zlib_compress: isize + 6 * (isize/1024
 * + 2) + 8 (no block is larger than its stored coding; blocks but the last
 * cover at least 1 KiB). */
int cz_zlib_bound(int isize);
/* deflate_inplace's zlib branch (CompressionEncoders.h:116-190, a
 * deflateInit(Z_DEFAULT_COMPRESSION) stream, SerializerIO_WaveletCompression_MPI_Simple.h:122)
 * on the GPU: one zlib stream (RFC 1950) of DEFLATE blocks (RFC 1951) of
 * up to 64 KiB each, every one dynamic Huffman, fixed Huffman or stored,
 * whichever is smallest, from an LZ77 parse with a 32 KiB window. Any zlib
 * inflate reads it; the bytes are not zlib's. isize < 2^24 - 64; cap >=
 * cz_zlib_bound(isize) always suffices. */
int cz_zlib_compress(cz_ctx *ctx, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out);
/* zdecompress's zlib branch (CompressionEncoders.h:48-88: inflateInit +
 * inflate(Z_FINISH)): a zlib stream (RFC 1950/1951) decoded on the GPU.
 * The Adler-32 trailer is checked; malformed or truncated input returns
 * CZ_E_CORRUPT (the reference accepts any non-zero inflate return). */
int cz_zlib_decompress(cz_ctx *ctx, const uint8_t *src, int isize, uint8_t *dst, int cap, int *out);

/* ---- field level (device buffers) ------------------------------------- */
/* Every device field pointer of this section and of the batch, plan and
 * refit calls (d_field, d_ref, d_fields[i]) must be 16-byte aligned: rows
 * are read and written as 16-byte vectors. Any cudaMalloc'd buffer is; an
 * offset view into one may not be. A misaligned pointer returns CZ_E_ARG
 * before any work is launched. */
/* Compress a field d_field[nz][ny][nx] (extents multiples of 32) into the
 * context's stream buffers. Asynchronous on `stream` except that it waits
 * for the stream's compressed size. Replaces the writer's _compress loop
 * (SerializerIO...:187-345) for one rank. */
int cz_field_compress(cz_ctx *ctx, const float *d_field, int nx, int ny, int nz, const cz_params *p, void *stream,
                      cz_stream *out);
/* Copy a compressed stream into caller-owned device buffers: d_data
 * (s->data_bytes bytes) and d_chunk_offsets (s->nchunks+1 entries, rebased
 * to start at 0). Either pointer may be NULL. */
int cz_stream_copy(cz_ctx *ctx, const cz_stream *s, uint8_t *d_data, long long *d_chunk_offsets, void *stream);
/* Decompress chunks (d_data, d_chunk_offsets[nchunks+1], device) holding
 * the records of the field's blocks in block order, blocks_per_chunk per
 * chunk, into d_field. The offsets must lie within d_data's buffer (as the
 * ones cz_stream_copy writes do; files go through the parser of
 * cz_decompress_image, which checks them); a chunk whose end precedes its
 * start, malformed chunks and malformed records are reported as
 * CZ_E_CORRUPT. */
int cz_field_decompress(cz_ctx *ctx, const uint8_t *d_data, const long long *d_chunk_offsets, int nchunks, int nx,
                        int ny, int nz, const cz_params *p, void *stream, float *d_field);

/* cz_field_decompress fused with cz2diff's error norms against a reference
 * field d_ref of the same extents (Tools/cz2diff.cpp:116-261): stats =
 * {e_inf, n_inf, e_1, n_1, e_2, n_2, min(ref), max(ref), n} with
 * e = |decoded - ref|, n = |ref| (e_2 and n_2 are sums of squares). The
 * differences and maxima are exact; sums are compensated per thread and
 * binary64 beyond (the reference sums serially in binary64). d_field may be
 * NULL (decode into context scratch). */
int cz_field_diff(cz_ctx *ctx, const uint8_t *d_data, const long long *d_chunk_offsets, int nchunks, int nx, int ny,
                  int nz, const cz_params *p, const float *d_ref, void *stream, float *d_field, double *stats);
/* cz2diff's RES line from those statistics and the compressed size
 * (CR, rel(e_inf), rel(e_1), mean(e_1), rel(e_2), mean(e_2), BPS, PSNR with
 * PSNR = 20 log10((max-min) / (2 sqrt(mse)))), same format. Host only. */
int cz_res_line(const double *stats, long long compressed_bytes, char *buf, int len);

/* The array layout of the reference's HDF5 tools: hdf2cz reads value
 * (gx,gy,gz) from in[ch + nch*(gz + nz*(gy + ny*gx))], z fastest, nch
 * interleaved channels (Tools/Test_IO_Compressed.h:192-217); cz2hdf writes
 * decoded blocks back in that order (Tools/cz2hdf.cpp:235-253). The codec's
 * field is x fastest, d_field[gz][gy][gx]. cz_field_from_zfastest takes
 * float (bytes = 4) or double (bytes = 8, rounded to nearest float) input;
 * cz_field_to_zfastest writes channel ch of a float array. Device buffers,
 * asynchronous on `stream`; ny <= 65535. */
int cz_field_from_zfastest(cz_ctx *ctx, const void *d_in, int bytes, int nch, int ch, int nx, int ny, int nz,
                           float *d_field, void *stream);
int cz_field_to_zfastest(cz_ctx *ctx, const float *d_field, int nx, int ny, int nz, int nch, int ch, float *d_out,
                         void *stream);

/* Many fields of uneven extents and thresholds in one persistent launch
 * (device work queue). eps[i] per field; p->eps is ignored. out[i]
 * describes field i's chunks inside the shared stream buffers. */
int cz_batch_compress(cz_ctx *ctx, int nfields, const float *const *d_fields, const int *dims /* 3*nfields: nx,ny,nz */,
                      const float *eps, const cz_params *p, void *stream, cz_stream *out);

/* ---- least-squares refit (device buffers) ----------------------------- */
/* The inverse transform as a linear operator and its adjoint, on nblocks
 * stacked 32^3 blocks (block g at +g*32768). Coefficients are in the
 * reference's positional layout (the array FullTransformEngine::fwt leaves
 * in place, FullWaveletTransform.h:44-49); samples are x fastest.
 * cz_iwt_linear evaluates FullTransformEngine::iwt (:51-56) in binary32
 * with its stencils as plain linear maps (not bit-exact to the reference's
 * binary64 stencils); cz_iwt_adjoint applies the exact transpose of that map
 * (the transposed 1D inverse operators in reverse sweep order). No
 * counterpart in the reference. Asynchronous on `stream`. */
int cz_iwt_linear(cz_ctx *ctx, const float *d_coef, long long nblocks, int wtype, float *d_blocks, void *stream);
int cz_iwt_adjoint(cz_ctx *ctx, const float *d_blocks, long long nblocks, int wtype, float *d_coef, void *stream);
/* cz_field_compress with the retained coefficients refit: the mask is the
 * plain path's (|c| > eps), the survivors minimise ||x - IWT(M c)||^2 per
 * block after `iters` (1..1000) CGLS steps started from the plain
 * survivors. Same stream layout, decoded by any reader of the plain
 * stream. No counterpart in the reference (whose threshold keeps the
 * forward coefficients, FullWaveletTransform.h:58-96). */
int cz_refit(cz_ctx *ctx, const float *d_field, int nx, int ny, int nz, const cz_params *p, int iters, void *stream,
             cz_stream *out);

/* ---- batch plans (device buffers) -------------------------------------- */
/* A batch of fields fixed once (device pointers, extents, thresholds) and
 * compressed many times: cz_plan_create sizes a private set of buffers,
 * optionally tunes the launch shape on the batch itself (tune != 0, timed
 * with CUDA events: the LZ4 stage's CTA width, 2, 4, 8 or 16 chunks per
 * CTA, then the wavelet kernel's row-prefetch variant; every shape writes
 * the same bytes), and captures the whole pipeline (one persistent wavelet
 * launch over every field's blocks through the device work queue, chunk
 * setup, scans, LZ4, gather) in a CUDA graph. cz_plan_launch is one graph
 * launch with no host work; the fields' contents may change between
 * launches. cz_plan_result waits for `stream` and describes the shared
 * stream (all) and, if per_field is not NULL, each field's chunks as in
 * cz_batch_compress. Records are one block per chunk. No counterpart in
 * the reference. */
typedef struct cz_plan cz_plan;
int cz_plan_create(cz_ctx *ctx, int nfields, const float *const *d_fields, const int *dims /* 3*nfields */,
                   const float *eps, const cz_params *p, int tune, cz_plan **out);
int cz_plan_launch(cz_plan *plan, void *stream);
int cz_plan_result(cz_plan *plan, void *stream, cz_stream *all, cz_stream *per_field);
int cz_plan_info(const cz_plan *plan, int *lz_warps, float *tune_ms /* 3: LZ4 ms at 2, 4, 8 */);
/* The tuned shape: shape[0] = LZ4 chunks per CTA, shape[1] = wavelet kernel
 * variant (0: the next block's rows load in two halves by the warps each
 * level leaves idle, 1: all at once after level 32); ms[0..3] = LZ4 stage at
 * 2, 4, 8, 16 chunks per CTA, ms[4..5] = wavelet kernel in variant 0, 1
 * (-1 where not timed). No counterpart in the reference. */
int cz_plan_shape(const cz_plan *plan, int *shape /* 2 */, float *ms /* 6 */);
const char *cz_plan_last_error(const cz_plan *plan);
int cz_plan_destroy(cz_plan *plan);

/* ---- allocation-free block compression (device buffers) --------------- */
/* No counterpart in the reference. For callers that cannot call cudaMalloc
 * (applications that hand all device memory to their own pool, pipelines
 * where an allocation would synchronise the device): compresses nblocks
 * (1..CZ_NOALLOC_MAX_BLOCKS) 32^3 blocks stacked in d_blocks (block g at
 * d_blocks + g*32768, x fastest) with the same encode kernel, using a
 * static device scratch array of the library (~2.2 MB per device, held
 * until exit) instead of allocating. Record g goes to d_records +
 * g*CZ_MAX_RECORD, its size to d_nbytes[g]; asynchronous on `stream`, on
 * the current device. The first call on a device looks up the scratch
 * address and should come before any stream capture. Calls share the
 * scratch, so calls that overlap on the GPU race. Returns CZ_E_ARG for
 * nblocks beyond the maximum, and when d_blocks is not 16-byte aligned or
 * d_records or d_nbytes is not 4-byte aligned (checked before any launch). */
#define CZ_NOALLOC_MAX_BLOCKS 16
int cz_blocks_compress_noalloc(const float *d_blocks, int nblocks, float eps, int wtype, int zerobits, int shuffle,
                               uint8_t *d_records, int *d_nbytes, void *stream);

/* ---- .cz files (host memory) ------------------------------------------ */
/* Several ranks writing one file (SerializerIO...:347-466). The grid of
 * bx x by x bz blocks is split into nranks z-slabs of bz/nranks block
 * layers; rank r compresses its slab (a field of nx x ny x nz/nranks) and
 * contributes its part: its chunks and the LUT of their offsets relative
 * to the part (cz_stream_part from a device stream, cz_part_write from host
 * chunks). Part r starts at cz_mini_bytes() plus the exclusive scan of the
 * parts' sizes (the writer's MPI_Exscan, :389); the mini header (at 0) and
 * the tail (header, BlockMetadata of every rank, HeaderLUT; at the end of
 * the last part) need every rank's part size and chunk count. All host
 * memory; no GPU work except cz_stream_part's copies. */
long long cz_mini_bytes(void);
int cz_mini_write(long long header_offset, uint8_t *out, long long cap);
long long cz_part_bytes(long long payload_bytes, int nchunks);
int cz_part_write(const uint8_t *payload, const long long *chunk_offsets /* nchunks+1, from 0 */, int nchunks,
                  uint8_t *out, long long cap, long long *written);
int cz_stream_part(cz_ctx *ctx, const cz_stream *s, uint8_t *out, long long cap, long long *written);
long long cz_tail_bytes(int bx, int by, int bz, int nranks, const cz_params *p);
int cz_tail_write(int bx, int by, int bz, int nranks, const long long *part_bytes, const int *part_chunks,
                  const cz_params *p, uint8_t *out, long long cap, long long *written);

/* Size of the .cz image for a compressed stream (header, metadata, LUT). */
long long cz_file_bytes(cz_ctx *ctx, const cz_stream *s, int nx, int ny, int nz, const cz_params *p);
/* Write the .cz image of `s` into host buffer out (capacity cap): the
 * reference writer's layout (SerializerIO...:347-466, 489-591) for one rank.
 * *written = image size. */
int cz_file_image(cz_ctx *ctx, const cz_stream *s, int nx, int ny, int nz, const cz_params *p, uint8_t *out,
                  long long cap, long long *written);
/* Host field in, .cz image out: H2D copy, compression, D2H copy and layout
 * in one call (the end-to-end drop-in for Write<channel>). */
int cz_compress_to_image(cz_ctx *ctx, const float *h_field, int nx, int ny, int nz, const cz_params *p,
                         void *stream, uint8_t *out, long long cap, long long *written);
/* Parse a .cz image: dims[3] (nx,ny,nz) and the encoder it declares. */
int cz_image_info(const uint8_t *img, long long size, int *dims, int *encoder);
/* .cz image in, host field out (the reader's load_file + load_block2 for
 * every block, Reader_WaveletCompression.h:255-754). wtype must match the
 * file's "Wavelets:" entry; shuffle is the build option the file was
 * written with (the format does not record it). */
int cz_decompress_image(cz_ctx *ctx, const uint8_t *img, long long size, int wtype, int shuffle, void *stream,
                        float *h_field, long long field_cap);

#ifdef __cplusplus
}
#endif
#endif
