/*
 * ref_harness.cpp -- C entry points around the reference's own codec, writer
 * and reader, compiled from the reference sources where they lie by
 * oracle/build_ref.py into oracle/_ref/libczref_<variant>.so.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing here is part of the product; the
 * reference headers are compiled unmodified, this file only provides the
 * grid/block/streamer types their templates expect (the roles played by
 * Cubism's Grid and Tools/Types_single.h in the reference build) and thin
 * extern "C" wrappers for ctypes.
 */
#include <mpi.h>

#include <algorithm>
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <time.h>
#include <vector>

typedef float Real;

#include "BlockInfo.h"

struct FluidElement { Real u; };

/* Block type with the accessors used by _compress (SerializerIO...:214-222). */
struct FluidBlock {
    static const int sizeX = _BLOCKSIZE_, sizeY = _BLOCKSIZE_, sizeZ = _BLOCKSIZE_;
    FluidElement data[_BLOCKSIZE_][_BLOCKSIZE_][_BLOCKSIZE_];
    FluidElement &operator()(int ix, int iy = 0, int iz = 0) { return data[iz][iy][ix]; }
};

/* Streamer: _compress takes the IterativeStreamer(b).operate(ix,iy,iz) path
 * for any name other than "StreamerGridPointIterative". */
struct FieldStreamer {
    static const int channels = 1;
    FluidBlock *ref;
    FieldStreamer() : ref(NULL) {}
    FieldStreamer(FluidBlock &b) : ref(&b) {}
    template <int channel> static Real operate(const FluidElement &e) { return e.u; }
    Real operate(int ix, int iy, int iz) const { return (*ref)(ix, iy, iz).u; }
    const char *name() { return "FieldStreamer"; }
};

/* Minimal single-rank grid with the interface SerializerIO uses. */
struct FieldGrid {
    int nb[3];
    std::vector<FluidBlock> blocks;
    std::vector<BlockInfo> infos;
    FieldGrid(int bx, int by, int bz) : blocks((size_t)bx * by * bz)
    {
        nb[0] = bx; nb[1] = by; nb[2] = bz;
        const int mx = std::max(bx, std::max(by, bz));
        const double h = 1.0 / mx;
        for (int iz = 0; iz < bz; ++iz)
            for (int iy = 0; iy < by; ++iy)
                for (int ix = 0; ix < bx; ++ix) {
                    const long long id = ix + (long long)bx * (iy + (long long)by * iz);
                    const int idx[3] = {ix, iy, iz};
                    const double org[3] = {ix * h, iy * h, iz * h};
                    infos.push_back(BlockInfo(id, idx, org, h, h / _BLOCKSIZE_, &blocks[id]));
                }
    }
    std::vector<BlockInfo> &getBlocksInfo() { return infos; }
    const std::vector<BlockInfo> &getBlocksInfo() const { return infos; }
    int getBlocksPerDimension(int d) const { return nb[d]; }
    int getResidentBlocksPerDimension(int d) const { return nb[d]; }
    double getH() const { return infos[0].h_gridpoint; }
    MPI_Comm getCartComm() const { return MPI_COMM_WORLD; }
    void fill(const float *field)
    {
        const int nx = nb[0] * _BLOCKSIZE_, ny = nb[1] * _BLOCKSIZE_;
        for (size_t b = 0; b < blocks.size(); ++b) {
            const int *ix = infos[b].index;
            for (int z = 0; z < _BLOCKSIZE_; ++z)
                for (int y = 0; y < _BLOCKSIZE_; ++y)
                    for (int x = 0; x < _BLOCKSIZE_; ++x)
                        blocks[b].data[z][y][x].u =
                            field[((size_t)(ix[2] * _BLOCKSIZE_ + z) * ny + (ix[1] * _BLOCKSIZE_ + y)) * nx +
                                  ix[0] * _BLOCKSIZE_ + x];
        }
    }
};

#include "SerializerIO_WaveletCompression_MPI_Simple.h"
#include "Reader_WaveletCompression.h"

typedef SerializerIO_WaveletCompression_MPI_SimpleBlocking<FieldGrid, FieldStreamer> Serializer;

/* The reference writer and reader print per call; silence fd 1 while they
 * run and restore it afterwards (the harness is loaded into test processes). */
struct QuietStdout {
    int saved;
    QuietStdout()
    {
        fflush(stdout);
        saved = dup(1);
        const int dn = open("/dev/null", O_WRONLY);
        dup2(dn, 1);
        close(dn);
    }
    ~QuietStdout()
    {
        fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
};

extern "C" {

/* WaveletCompressor::compress on one block (WaveletCompressor.cpp:152-182). */
int ref_block_compress(const float *in, float eps, int wtype, unsigned char *out, int *nbytes)
{
    WaveletCompressor *c = new WaveletCompressor;
    memcpy(&c->uncompressed_data()[0][0][0], in, sizeof(float) * _BLOCKSIZE_ * _BLOCKSIZE_ * _BLOCKSIZE_);
    const int nb = (int)c->compress(eps, false, wtype);
    memcpy(out, c->compressed_data(), nb);
    *nbytes = nb;
    delete c;
    return 0;
}

/* WaveletCompressor::decompress on one record (WaveletCompressor.cpp:231-259). */
int ref_block_decompress(const unsigned char *in, int nbytes, int wtype, float *out)
{
    WaveletCompressor *c = new WaveletCompressor;
    memcpy(c->compressed_data(), in, nbytes);
    c->decompress(false, nbytes, wtype, *(Real(*)[_BLOCKSIZE_][_BLOCKSIZE_][_BLOCKSIZE_])out);
    delete c;
    return 0;
}

/* The forward transform alone (FullTransform::fwt), for coefficient parity. */
void ref_fwt(float *block, int wtype)
{
    WaveletsOnInterval::FullTransform<_BLOCKSIZE_> *t = new WaveletsOnInterval::FullTransform<_BLOCKSIZE_>;
    memcpy(t->data, block, sizeof(t->data));
    t->fwt(wtype);
    memcpy(block, t->data, sizeof(t->data));
    delete t;
}

void ref_iwt(float *block, int wtype)
{
    WaveletsOnInterval::FullTransform<_BLOCKSIZE_> *t = new WaveletsOnInterval::FullTransform<_BLOCKSIZE_>;
    memcpy(t->data, block, sizeof(t->data));
    t->iwt(wtype);
    memcpy(block, t->data, sizeof(t->data));
    delete t;
}

#if defined(_USE_LZ4_)
int ref_lz4_compress(const char *src, char *dst, int isize) { return LZ4_compress(src, dst, isize); }
int ref_lz4_decompress(const char *src, char *dst, int isize, int cap)
{
    return LZ4_uncompress_unknownOutputSize(src, dst, isize, cap);
}
#endif

/* The lossless stage exactly as the writer calls it (CompressionEncoders.h:113-247). */
int ref_deflate_inplace(unsigned char *buf, unsigned len, unsigned cap)
{
    z_stream s;
    memset(&s, 0, sizeof(s));
    deflateInit(&s, Z_DEFAULT_COMPRESSION);
    unsigned mah = cap;
    const int err = deflate_inplace(&s, buf, len, &mah);
    const int out = (int)s.total_out;
    deflateEnd(&s);
    return err == Z_OK ? out : -1;
}

/* Full writer: Write<0> of a field (x-fastest [nz][ny][nx]) into a .cz file.
 * With path == NULL the file write is skipped (CUBISMZ_NOIO, :606) and the
 * call times the reference's compress+serialization. Returns seconds. */
double ref_write_cz(const float *field, int nx, int ny, int nz, float eps, int wtype, const char *path,
                    int nthreads, int repeats)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    FieldGrid *g = new FieldGrid(nx / _BLOCKSIZE_, ny / _BLOCKSIZE_, nz / _BLOCKSIZE_);
    g->fill(field);
    Serializer *w = new Serializer;
    w->set_threshold(eps);
    w->set_wtype_write(wtype);
    if (path == NULL) setenv("CUBISMZ_NOIO", "1", 1);
    else unsetenv("CUBISMZ_NOIO");
    QuietStdout quiet;
    double best = 1e30;
    for (int r = 0; r < (repeats > 0 ? repeats : 1); ++r) {
        if (path) remove(path);
        timespec a, b;
        clock_gettime(CLOCK_MONOTONIC, &a);
        w->Write<0>(*g, path ? std::string(path) : std::string("/dev/null"));
        clock_gettime(CLOCK_MONOTONIC, &b);
        const double dt = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
        if (dt < best) best = dt;
    }
    delete w;
    delete g;
    return best;
}

/* Full reader: load_file + load_block2 for every block (the cz2hdf decode
 * path, Tools/cz2hdf.cpp:92-98,229). Writes the field x-fastest. */
int ref_read_cz(const char *path, int wtype, float *field, int *dims)
{
    QuietStdout quiet;
    Reader_WaveletCompressionMPI *r = new Reader_WaveletCompressionMPI(MPI_COMM_WORLD, path, 0, wtype);
    r->load_file();
    const int bx = r->xblocks(), by = r->yblocks(), bz = r->zblocks();
    dims[0] = bx * _BLOCKSIZE_;
    dims[1] = by * _BLOCKSIZE_;
    dims[2] = bz * _BLOCKSIZE_;
    if (field) {
        static Real blk[_BLOCKSIZE_][_BLOCKSIZE_][_BLOCKSIZE_];
        const int nx = dims[0], ny = dims[1];
        for (int iz = 0; iz < bz; ++iz)
            for (int iy = 0; iy < by; ++iy)
                for (int ix = 0; ix < bx; ++ix) {
                    r->load_block2(ix, iy, iz, blk);
                    for (int z = 0; z < _BLOCKSIZE_; ++z)
                        for (int y = 0; y < _BLOCKSIZE_; ++y)
                            memcpy(field + ((size_t)(iz * _BLOCKSIZE_ + z) * ny + (iy * _BLOCKSIZE_ + y)) * nx +
                                       ix * _BLOCKSIZE_,
                                   blk[z][y], sizeof(Real) * _BLOCKSIZE_);
                }
    }
    delete r;
    return 0;
}

int ref_entries_per_chunk(void) { return (int)((4 * 1024 * 1024) / (sizeof(WaveletCompressor) + sizeof(int))); }
int ref_sizeof_compressor(void) { return (int)sizeof(WaveletCompressor); }
}
