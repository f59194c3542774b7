/*
 * czoracle.h -- CPU oracle for the CubismZ wavelet block codec.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * algorithm (fab4100/CubismZ, Compressor/source) that tests/ and
 * __graft_entry__.smoke() check the GPU results against and bench.py's CPU
 * baseline leg runs. The product path (libczgpu.so) never links, loads or
 * calls it.
 *
 * Parity pinning: the restatement is checked bit-for-bit against the
 * reference's own sources compiled in oracle/_ref (oracle/build_ref.py) on
 * seeded inputs, and against the reference's published golden line
 * Tests/Test1/cselab_ref_run_all.txt:12 (demo.h5, wtype 3, thr 5e-5, zlib).
 *
 * Layouts:
 *   block    float[32][32][32], x fastest (data[z][y][x]) as in
 *            WaveletCompressor::uncompressed_data() (WaveletCompressor.h:57).
 *   record   [4096-byte LSB-first significance mask][S survivors * 4 bytes]
 *            (WaveletCompressor.cpp:152-182).
 */
#ifndef CZORACLE_H
#define CZORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CZO_BS 32
#define CZO_BS3 (32 * 32 * 32)
#define CZO_MASKBYTES 4096
#define CZO_MAXRECORD (CZO_MASKBYTES + 4 * CZO_BS3)

/* 1D transform of one line of n floats (n in {8,16,32}); fwd != 0 forward. */
void czo_transform1d(float *line, int n, int wtype, int fwd);

/* Multilevel 3D transform of one block in place (positional layout). */
void czo_fwt(float *block, int wtype);
void czo_iwt(float *block, int wtype);

/* Threshold: mask bits (one byte per bit, 0/1) in positional order and the
 * survivors in coarse-first stream order. Returns the survivor count. */
int czo_threshold(const float *block, float eps, uint8_t *mask_bits, float *survivors);

/* Whole per-block codec, byte-compatible with WaveletCompressor::compress
 * (zerobits: 0 or n low mantissa bits cleared; shuffle: 0/1). Returns 0. */
int czo_block_compress(const float *in, float eps, int wtype, int zerobits, int shuffle,
                       uint8_t *out, int *nbytes);
/* Returns 0 on success, negative on a malformed record. */
int czo_block_decompress(const uint8_t *in, int nbytes, int wtype, int shuffle, float *out);

/* FP64 restatement of the same transform (quality oracle). */
void czo_fwt_f64(double *block, int wtype);
void czo_iwt_f64(double *block, int wtype);
/* explicit inverse line operator (row-major n x n) and the adjoint of czo_iwt_f64 */
void czo_inv_matrix(int n, int wtype, double *M);
void czo_iwt_adj_f64(double *block, int wtype);

/* LZ4 legacy block format. Decoder semantics and error conventions follow
 * LZ4_uncompress_unknownOutputSize (ThirdParty/lz4/lz4.c:802-905): returns
 * the decoded length, or minus the input position of the error (the
 * reference decoder's values, pinned by tests/golden/lz4_cases.json). */
int czo_lz4_decompress(const uint8_t *src, int isize, uint8_t *dst, int cap);
/* LZ4_compress (ThirdParty/lz4/lz4.c:337-700) restated: the reference's
 * bytes, pinned against its build and the committed chunks. Returns bytes
 * written. */
int czo_lz4_compress(const uint8_t *src, int isize, uint8_t *dst, int cap);
int czo_lz4_bound(int isize);

/* Field-level compression, CPU (OpenMP when built with it): the reference's
 * _compress loop (SerializerIO_WaveletCompression_MPI_Simple.h:187-345).
 * field is x-fastest [nz][ny][nx], all multiples of 32. Chunks hold
 * blocks_per_chunk consecutive records; encoder 0 = none, 1 = lz4.
 * out receives the concatenated chunks; chunk_off[nchunks+1] their offsets;
 * returns total bytes or negative on overflow. */
long long czo_field_compress(const float *field, int nx, int ny, int nz, float eps, int wtype,
                             int zerobits, int shuffle, int encoder, int blocks_per_chunk,
                             int nthreads, uint8_t *out, long long cap, long long *chunk_off);
/* Inverse of czo_field_compress. Returns 0 or negative on error. */
int czo_field_decompress(const uint8_t *data, const long long *chunk_off, int nchunks,
                         int nx, int ny, int nz, int wtype, int shuffle, int encoder,
                         int blocks_per_chunk, int nthreads, float *field);

int czo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
