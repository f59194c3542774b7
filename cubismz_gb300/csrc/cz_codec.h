// cz_codec.h -- internal interface between the C-ABI layer and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// One field of a (possibly batched) launch, x fastest [nz][ny][nx], all
// extents multiples of 32. block0 is the global index of the field's first
// block; blocks of a field are numbered ix fastest, then iy, iz (the
// reference grid's order, Grid.h:81-90).
struct CzField {
    const float *data;
    int nx, ny, nz;
    float eps;
    long long block0;
};

extern "C" int cz_codec_smem_bytes(void);

// variant 0: the next block's rows load in two halves, by the warps each
// level leaves idle; 1: all at once after level 32 (same records)
cudaError_t cz_launch_encode(int wtype, const CzField *fields, int nfields, long long total_blocks, int zerobits,
                             int shuffle, uint8_t *stage, int *rec_bytes, unsigned long long *queue, int grid,
                             cudaStream_t st, int variant = 0);
// Record of block g at base + rec_off[g] ([int32 nbytes][record]); a
// negative rec_off marks a block whose record is missing (status -1).
// diff_ref (optional, a field of the same geometry as fields[0]): per-block
// error statistics into diff_out[8*g] (cz2diff's quantities).
// Byte planes 1 and 2 of one-record chunks left in the LZ4 input by
// cz_launch_lz4_decode (hole per chunk = per block, chunk c at src +
// src_off[c]); hole == nullptr: every record is whole.
struct CzPlanes {
    const int4 *hole = nullptr;
    const uint8_t *src = nullptr;
    const long long *src_off = nullptr;
};
cudaError_t cz_launch_decode(int wtype, const CzField *fields, int nfields, long long total_blocks, int shuffle,
                             const uint8_t *base, const long long *rec_off, int *status, unsigned long long *queue,
                             int grid, cudaStream_t st, const float *diff_ref = nullptr, double *diff_out = nullptr,
                             CzPlanes planes = CzPlanes());
cudaError_t cz_launch_diff_total(const double *per_block, long long nblocks, double *total, cudaStream_t st);

// Linear inverse transform and its adjoint on stacked 32^3 blocks; block
// coefficients in the reference's positional layout, samples x fastest
// (cz_refit.cu).
cudaError_t cz_launch_iwt_linear(int wtype, const float *coef, float *out, long long nblocks, int grid,
                                 cudaStream_t st);
cudaError_t cz_launch_iwt_adjoint(int wtype, const float *in, float *coef, long long nblocks, int grid,
                                  cudaStream_t st);
// Encode with the least-squares refit of the survivors (iters CGLS steps per
// block under the plain mask); scratch holds cz_refit_scratch_floats(grid).
size_t cz_refit_scratch_floats(int grid);
cudaError_t cz_launch_refit(int wtype, const CzField *fields, int nfields, long long total_blocks, int zerobits,
                            int shuffle, int iters, uint8_t *stage, int *rec_bytes, unsigned long long *queue,
                            float *scratch, int grid, cudaStream_t st);

// LZ4 stage (cz_lz4.cu). Chunk c's input is in[in_off[c] .. in_off[c]+in_len[c]);
// the encoder reads it as aligned words, so in + in_off[c] must be a multiple
// of 4 bytes (records and the staged host inputs are), and reads up to 64
// bytes past its end (buffers carry tail room). Outputs may start anywhere.
// records != 0: chunks hold block records with shuffled byte planes; the
// search skips planes 1 and 2 (copied as literals).
// warps: 2, 4, 8 or 16 warps (chunks) per CTA (16 takes an SM); any
// choice gives the same bytes (the parse's super-window, 512 or 768
// positions, follows from nchunks and the SM count alone).
// hole (optional): written for every chunk, {out position, input position,
// length, 0} of one literal-only span (byte planes 1 and 2 of a record
// chunk) that the encoder leaves unwritten in its output for the gather to
// copy from the input; length 0 when there is none.
// effort: 0 the lane-parallel parse alone; 1 (default) also extends matches
// backwards over equal bytes and keeps the tail of a match that a lower
// lane's match overlaps; 2 also takes repeats at distance 1-3 that the hash
// table misses and starts each lane's walk 8 positions early.
cudaError_t cz_launch_lz4_encode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, int *out_len, int records, int warps,
                                 int grid, cudaStream_t st, int4 *hole = nullptr, int effort = 1);
// The LZ77 parse of the LZ4 encoder for DEFLATE: distances up to 32 KiB,
// 8-byte sequence records (zl::seq_pack) per chunk at seq + seq_off[c]
// (capacity 8 * (in_len/4 + 2) bytes); seq_bytes[c] = record bytes.
cudaError_t cz_launch_lz77_parse(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *seq, const long long *seq_off, int *seq_bytes, int records, int grid,
                                 cudaStream_t st, int effort = 1);
// zlib streams (RFC 1950/1951) from the parse: chunk c at out + c * out_slot
// (out_slot >= cz_zlib_bound of the chunk), out_off[c] = c * out_slot,
// out_len[c] = stream bytes, -1 for a bad parse, -2..-4 for an internal
// inconsistency (never written past the slot).
// records: chunks of shuffled block records (blocks end at mask and planes).
cudaError_t cz_launch_deflate(const uint8_t *in, const long long *in_off, const int *in_len, const uint8_t *seq,
                              const long long *seq_off, const int *seq_bytes, int nchunks, int records,
                              uint8_t *out, long long out_slot, long long *out_off, int *out_len, int grid,
                              cudaStream_t st);
// hole (optional; one-record chunks of shuffled records only): written for
// every chunk; {out position, input position, length, 0} of the record's
// byte planes 1 and 2 when one literal run covers them whole -- the decoder
// then leaves that span of its output unwritten and the record's reader
// takes it from the input (CzPlanes); length 0 otherwise.
cudaError_t cz_launch_lz4_decode(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks,
                                 uint8_t *out, const long long *out_off, const int *out_cap, int *out_len, int grid,
                                 cudaStream_t st, int4 *hole = nullptr);

// Stream assembly helpers (cz_lz4.cu, cz_stream.cu)
// With hole (from cz_launch_lz4_encode): the span of each chunk that the
// encoder left unwritten comes from hsrc + hsrc_off[c] + hole[c].y.
cudaError_t cz_launch_gather(const uint8_t *src, const long long *src_off, const int *len, int nchunks,
                             uint8_t *dst, const long long *dst_off, cudaStream_t st, const int4 *hole = nullptr,
                             const uint8_t *hsrc = nullptr, const long long *hsrc_off = nullptr);
// Chunk layout of the encode side: chunk c holds blocks [c*bpc, (c+1)*bpc).
// Fills in_off/in_len (chunk inputs in chunk_in, or in the slots when bpc=1),
// blk_dst (where block g's [nbytes][record] goes inside chunk_in) and lz_off.
cudaError_t cz_launch_chunk_setup(int bpc, long long nblocks, int nchunks, const int *rec_bytes, long long *in_off,
                                  int *in_len, long long *blk_dst, long long *lz_off, long long lz_slot,
                                  cudaStream_t st);
// Copies block g's [nbytes][record] from its slot to chunk_in + blk_dst[g].
cudaError_t cz_launch_pack_records(const uint8_t *stage, const int *rec_bytes, long long nblocks,
                                   const long long *blk_dst, uint8_t *chunk_in, cudaStream_t st);
// Exclusive scan of len[0..n) into off[0..n], off[n] = total (n <= 2^31).
cudaError_t cz_launch_scan(const int *len, int n, long long *off, cudaStream_t st);
// The same starting from the value already in off[0] (a running total).
cudaError_t cz_launch_scan_from(const int *len, int n, long long *off, cudaStream_t st);
// Decode side: walks the [nbytes] headers of each decoded chunk (chunk c at
// base + c*chunk_cap, dec_len[c] bytes) and records where every block's
// record starts (rec_off, relative to base); -1 and status -1 on a short or
// malformed chunk. src_off/src_len, if not NULL, give raw (not LZ4) chunks.
cudaError_t cz_launch_locate_records(int bpc, long long nblocks, int nchunks, const long long *chunk_base,
                                     const int *dec_len, long long *rec_off, int *status, const uint8_t *base,
                                     cudaStream_t st);
cudaError_t cz_launch_decode_setup(int nchunks, const long long *off, int *in_len, long long *dec_off, int *dec_cap,
                                   long long cap, int raw, cudaStream_t st);
cudaError_t cz_launch_chunk_records(int nchunks, int maxsub, const long long *chunk_base, const int *dec_len,
                                    const uint8_t *base, long long *chunk_rec, cudaStream_t st);
cudaError_t cz_launch_map_blocks(long long nblocks, int nchunks, int maxsub, const int *block_chunk,
                                 const int *block_subid, const long long *chunk_rec, long long *rec_off,
                                 cudaStream_t st);
cudaError_t cz_launch_status_reduce(const int *status, long long n, int *flag, cudaStream_t st);
cudaError_t cz_launch_neg_reduce(const int *v, int n, int *flag, cudaStream_t st);
cudaError_t cz_launch_rebase(long long *off, int n, long long base, cudaStream_t st);

// Layout of the reference's HDF5 tools (cz_ingest.cu): z-fastest arrays with
// interleaved channels <-> the x-fastest field. bytes: 4 (float) or 8 (double).
cudaError_t cz_launch_from_zfastest(const void *in, int bytes, int nch, int ch, int nx, int ny, int nz, float *out,
                                    cudaStream_t st, int *err = nullptr,
                                    bool *used_tma = nullptr);
cudaError_t cz_launch_to_zfastest(const float *in, int nx, int ny, int nz, int nch, int ch, float *out,
                                  cudaStream_t st, int *err = nullptr,
                                  bool *used_tma = nullptr);

// zlib streams (cz_zlib.cu): one warp per chunk; out_len[c] = bytes or < 0.
cudaError_t cz_launch_inflate(const uint8_t *in, const long long *in_off, const int *in_len, int nchunks, uint8_t *out,
                              const long long *out_off, const int *out_cap, int *out_len, int grid, cudaStream_t st);
