// cz_format.cpp -- the .cz container, host side.
//
// Layout written by the reference for one rank
// (SerializerIO_WaveletCompression_MPI_Simple.h:347-466, 489-591):
//   [size_t header_offset][binary-ocean title]
//   [chunk payloads back to back][size_t LUT: chunk offsets within the rank data]
//   [ASCII header][BlockMetadata x nblocks][binary-LUT title][HeaderLUT]
// BlockMetadata = {int idcompression, subid, ix, iy, iz} packed (20 bytes),
// HeaderLUT = {size_t aggregate_bytes (payloads + LUT), int nchunks} packed
// (12 bytes) (WaveletSerializationTypes.h:16-18). The titles and header keys
// are format constants the reader matches (Reader_WaveletCompression.h:255-560),
// so they are spelled exactly as the reference spells them.
#include "cz_format.h"

#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

namespace czf {

static const char *kOceanTitle = "\n==============START-BINARY-OCEAN==============\n";
static const char *kLutTitle = "\n==============START-BINARY-LUT==============\n";

// FullWaveletTransform.h:28-35
const char *wavelet_name(int wtype)
{
    if (wtype == 0) return "None";
    if (wtype == 1) return "InterpWavelet4thOrder";
    if (wtype == 2) return "LiftedInterpWavelet4thOrder";
    if (wtype == 3) return "AverageInterpWavelet3rdOrder";
    return "None";
}

static const char *encoder_name(int enc) { return enc == 1 ? "lz4" : (enc == 2 ? "zlib" : "none"); }

// The header text of SerializerIO...:495-556, formatted with the same
// iostream defaults (the threshold is a float, the extents doubles). Blocks
// is the whole grid, SubdomainBlocks one rank's share.
std::string header_text_sub(int bx, int by, int bz, int sbx, int sby, int sbz, float threshold, int wtype,
                            int encoder)
{
    const int mx = std::max(bx, std::max(by, bz));
    const double h = (1.0 / mx) / 32;  // Grid spacing of a unit-extent grid (Grid.h:75-90)
    std::stringstream ss;
    ss << "\n==============START-ASCI-HEADER==============\n";
    ss << "Endianess: " << "little" << "\n";
    ss << "sizeofReal: " << 4 << "\n";
    ss << "sizeofsize_t: " << 8 << "\n";
    ss << "sizeofBlockMetadata: " << 20 << "\n";
    ss << "sizeofHeaderLUT: " << 12 << "\n";
    ss << "sizeofCompressedBlock: " << 20 << "\n";
    ss << "Blocksize: " << 32 << "\n";
    ss << "Blocks: " << bx << " x " << by << " x " << bz << "\n";
    ss << "Extent: " << h * bx * 32 << " " << h * by * 32 << " " << h * bz * 32 << "\n";
    ss << "SubdomainBlocks: " << sbx << " x " << sby << " x " << sbz << "\n";
    ss << "HalfFloat: " << "no" << "\n";
    ss << "Wavelets: " << wavelet_name(wtype) << "\n";
    ss << "WaveletThreshold: " << threshold << "\n";
    ss << "Encoder: " << encoder_name(encoder) << "\n";
    ss << "==============START-BINARY-METABLOCKS==============\n";
    return ss.str();
}

std::string header_text(int bx, int by, int bz, float threshold, int wtype, int encoder)
{
    return header_text_sub(bx, by, bz, bx, by, bz, threshold, wtype, encoder);
}

long long mini_header_bytes() { return 8 + (long long)strlen(kOceanTitle); }

long long image_bytes(long long payload, int nchunks, long long nblocks, const std::string &header)
{
    return 8 + (long long)strlen(kOceanTitle) + payload + 8LL * nchunks + (long long)header.size() + 20LL * nblocks +
           (long long)strlen(kLutTitle) + 12;
}

template <class T>
static void put(uint8_t *&p, const T &v)
{
    memcpy(p, &v, sizeof(T));
    p += sizeof(T);
}

long long write_image(uint8_t *out, const uint8_t *payload, long long payload_bytes, const long long *chunk_off,
                      int nchunks, const int *block_chunk, const int *block_subid, int bx, int by, int bz,
                      const std::string &header)
{
    uint8_t *p = out;
    const long long mini = 8 + (long long)strlen(kOceanTitle);
    const long long aggregate = payload_bytes + 8LL * nchunks;
    const unsigned long long header_off = (unsigned long long)(mini + aggregate);
    put(p, header_off);
    memcpy(p, kOceanTitle, strlen(kOceanTitle));
    p += strlen(kOceanTitle);
    if (payload != p) memmove(p, payload, (size_t)payload_bytes);
    p += payload_bytes;
    for (int c = 0; c < nchunks; ++c) put(p, (unsigned long long)chunk_off[c]);
    memcpy(p, header.data(), header.size());
    p += header.size();
    const long long nblocks = (long long)bx * by * bz;
    for (long long g = 0; g < nblocks; ++g) {
        const int ix = (int)(g % bx), iy = (int)((g / bx) % by), iz = (int)(g / ((long long)bx * by));
        put(p, block_chunk[g]);
        put(p, block_subid[g]);
        put(p, ix);
        put(p, iy);
        put(p, iz);
    }
    memcpy(p, kLutTitle, strlen(kLutTitle));
    p += strlen(kLutTitle);
    put(p, (unsigned long long)aggregate);
    put(p, nchunks);
    return (long long)(p - out);
}

static bool read_line(const uint8_t *img, long long size, long long &pos, std::string &line)
{
    line.clear();
    while (pos < size) {
        const char c = (char)img[pos++];
        line.push_back(c);
        if (c == '\n') return true;
    }
    return false;
}

static bool key_value(const std::string &line, const char *key, std::string &val)
{
    const size_t n = strlen(key);
    if (line.compare(0, n, key) != 0) return false;
    size_t i = n;
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
    val = line.substr(i);
    while (!val.empty() && (val.back() == '\n' || val.back() == '\r' || val.back() == ' ')) val.pop_back();
    return true;
}

// Reader_WaveletCompression::load_file (Reader_WaveletCompression.h:255-560):
// header fields, block metadata, per-subdomain LUTs -> chunk geometry.
int parse_image(const uint8_t *img, long long size, Parsed &out, std::string &err)
{
    const long long mini = 8 + (long long)strlen(kOceanTitle);
    if (size < mini) {
        err = "file shorter than the mini header";
        return -1;
    }
    unsigned long long hoff;
    memcpy(&hoff, img, 8);
    if ((long long)hoff < mini || (long long)hoff >= size) {
        err = "header offset out of range";
        return -1;
    }
    long long pos = (long long)hoff;
    std::string line, v;
    read_line(img, size, pos, line);  // "\n"
    read_line(img, size, pos, line);
    if (line != "==============START-ASCI-HEADER==============\n") {
        err = "missing ASCII header";
        return -1;
    }
    out = Parsed();
    int sub[3] = {-1, -1, -1};
    for (;;) {
        if (!read_line(img, size, pos, line)) {
            err = "truncated header";
            return -1;
        }
        if (line == "==============START-BINARY-METABLOCKS==============\n") break;
        if (key_value(line, "Endianess:", v)) {
            if (v != "little") {
                err = "big-endian files are not supported";
                return -1;
            }
        } else if (key_value(line, "sizeofReal:", v)) {
            if (v != "4") { err = "sizeofReal is not 4"; return -1; }
        } else if (key_value(line, "sizeofsize_t:", v)) {
            if (v != "8") { err = "sizeofsize_t is not 8"; return -1; }
        } else if (key_value(line, "Blocksize:", v)) {
            if (v != "32") { err = "block size is not 32"; return -1; }
        } else if (key_value(line, "Blocks:", v)) {
            if (sscanf(v.c_str(), "%d x %d x %d", &out.bx, &out.by, &out.bz) != 3) { err = "bad Blocks"; return -1; }
        } else if (key_value(line, "SubdomainBlocks:", v)) {
            if (sscanf(v.c_str(), "%d x %d x %d", &sub[0], &sub[1], &sub[2]) != 3) {
                err = "bad SubdomainBlocks";
                return -1;
            }
        } else if (key_value(line, "HalfFloat:", v)) {
            if (v != "no") { err = "half-float files are not supported"; return -1; }
        } else if (key_value(line, "Wavelets:", v)) {
            out.wavelets = v;
        } else if (key_value(line, "WaveletThreshold:", v)) {
            out.threshold = (float)atof(v.c_str());
        } else if (key_value(line, "Encoder:", v)) {
            out.encoder = v == "lz4" ? 1 : (v == "zlib" ? 2 : (v == "none" ? 0 : -1));
        }
    }
    if (out.bx <= 0 || out.by <= 0 || out.bz <= 0 || sub[0] <= 0 || sub[1] <= 0 || sub[2] <= 0) {
        err = "missing block counts";
        return -1;
    }
    // every block takes 20 bytes of metadata, which bounds the products
    // below before they are formed; a subdomain is no larger than the grid
    const long long room = (size - pos) / 20;
    if (out.bx > room || out.by > room / out.bx || out.bz > room / ((long long)out.bx * out.by)) {
        err = "truncated block metadata";
        return -1;
    }
    if (sub[0] > out.bx || sub[1] > out.by || sub[2] > out.bz) {
        err = "SubdomainBlocks larger than Blocks";
        return -1;
    }
    const long long nblocks = (long long)out.bx * out.by * out.bz;
    const long long bps = (long long)sub[0] * sub[1] * sub[2];
    if (nblocks % bps) {
        err = "subdomain blocks do not divide the grid";
        return -1;
    }
    const long long nsub = nblocks / bps;
    std::vector<int> meta(5 * nblocks);
    memcpy(meta.data(), img + pos, (size_t)(20 * nblocks));
    pos += 20 * nblocks;
    pos += 1;  // fgetc of the title's leading newline
    read_line(img, size, pos, line);
    if (line != "==============START-BINARY-LUT==============\n") {
        err = "missing LUT title";
        return -1;
    }
    if (pos + 12 * nsub > size) {
        err = "truncated HeaderLUT";
        return -1;
    }
    out.chunk_start.clear();
    out.chunk_size.clear();
    long long base = mini;
    std::vector<long long> first_chunk(nsub);
    std::vector<int> sub_chunks(nsub);
    for (long long s = 0; s < nsub; ++s) {
        unsigned long long agg;
        int nch;
        memcpy(&agg, img + pos + 12 * s, 8);
        memcpy(&nch, img + pos + 12 * s + 8, 4);
        // agg bytes of this subdomain lie between base and the header, and
        // end in its LUT of nch offsets (compared without forming base + agg)
        if (nch <= 0 || agg > (unsigned long long)(hoff - base) || agg < 8ULL * (unsigned long long)nch) {
            err = "bad HeaderLUT";
            return -1;
        }
        first_chunk[s] = (long long)out.chunk_start.size();
        sub_chunks[s] = nch;
        const unsigned long long data = agg - 8ULL * (unsigned long long)nch;  // chunk bytes before the LUT
        std::vector<unsigned long long> lut(nch);
        memcpy(lut.data(), img + base + (long long)data, 8 * (size_t)nch);
        for (int i = 0; i < nch; ++i) {
            const unsigned long long end = (i + 1 < nch) ? lut[i + 1] : data;
            if (lut[i] >= end || end > data) {
                err = "chunk LUT not increasing within the subdomain";
                return -1;
            }
            out.chunk_start.push_back(base + (long long)lut[i]);
            out.chunk_size.push_back((long long)(end - lut[i]));
        }
        base += (long long)agg;
    }
    if (base != (long long)hoff) {
        err = "subdomain data does not end at the header";
        return -1;
    }
    // block (ix,iy,iz) -> (chunk, subid); metadata chunk ids are per subdomain
    out.block_chunk.assign(nblocks, -1);
    out.block_subid.assign(nblocks, -1);
    out.max_subid = 0;
    for (long long i = 0; i < nblocks; ++i) {
        const int *m = &meta[5 * i];
        const long long s = i / bps;
        const int ix = m[2], iy = m[3], iz = m[4];
        // a chunk holds at most its subdomain's blocks: a larger record index
        // (subid) is damage, and would size the decode buffers by it
        if (ix < 0 || iy < 0 || iz < 0 || ix >= out.bx || iy >= out.by || iz >= out.bz || m[0] < 0 || m[1] < 0 ||
            m[1] >= bps) {
            err = "bad block metadata";
            return -1;
        }
        const long long gc = first_chunk[s] + m[0];
        if (m[0] >= sub_chunks[s]) {
            err = "block metadata names a missing chunk";
            return -1;
        }
        const long long g = ix + (long long)out.bx * (iy + (long long)out.by * iz);
        out.block_chunk[g] = (int)gc;
        out.block_subid[g] = m[1];
        if (m[1] + 1 > out.max_subid) out.max_subid = m[1] + 1;
    }
    for (long long g = 0; g < nblocks; ++g)
        if (out.block_chunk[g] < 0) {
            err = "a block has no metadata";
            return -1;
        }
    return 0;
}

// ------------------------------------------------ several ranks, one file
// The writer's collective layout (SerializerIO...:371-466): rank r's data
// (its chunks, then its LUT of chunk offsets relative to the rank's data)
// starts at the mini header plus the exclusive scan of the ranks' data sizes
// (MPI_Exscan, :389); the header, the ranks' BlockMetadata in rank order and
// the HeaderLUT of every rank follow the last rank's data.
long long write_part(uint8_t *out, const uint8_t *payload, long long payload_bytes, const long long *chunk_off,
                     int nchunks)
{
    uint8_t *p = out;
    if (payload != p) memmove(p, payload, (size_t)payload_bytes);
    p += payload_bytes;
    for (int c = 0; c < nchunks; ++c) put(p, (unsigned long long)chunk_off[c]);
    return (long long)(p - out);
}

void write_mini(uint8_t *out, long long header_offset)
{
    uint8_t *p = out;
    put(p, (unsigned long long)header_offset);
    memcpy(p, kOceanTitle, strlen(kOceanTitle));
}

long long tail_bytes(long long nblocks, int nranks, const std::string &header)
{
    return (long long)header.size() + 20LL * nblocks + (long long)strlen(kLutTitle) + 12LL * nranks;
}

// Ranks own z-slabs of bz / nranks block layers; blocks_per_chunk records
// per chunk in each rank's block order (ix fastest).
long long write_tail(uint8_t *out, const std::string &header, int bx, int by, int bz, int nranks, int bpc,
                     const long long *part_bytes, const int *part_chunks)
{
    uint8_t *p = out;
    memcpy(p, header.data(), header.size());
    p += header.size();
    const int sbz = bz / nranks;
    const long long bps = (long long)bx * by * sbz;
    for (int r = 0; r < nranks; ++r)
        for (long long l = 0; l < bps; ++l) {
            put(p, (int)(l / bpc));
            put(p, (int)(l % bpc));
            put(p, (int)(l % bx));
            put(p, (int)((l / bx) % by));
            put(p, (int)(r * sbz + l / ((long long)bx * by)));
        }
    memcpy(p, kLutTitle, strlen(kLutTitle));
    p += strlen(kLutTitle);
    for (int r = 0; r < nranks; ++r) {
        put(p, (unsigned long long)part_bytes[r]);
        put(p, part_chunks[r]);
    }
    return (long long)(p - out);
}

}  // namespace czf
