// cz_format.h -- .cz container helpers (host).
#pragma once
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

namespace czf {

const char *wavelet_name(int wtype);
std::string header_text(int bx, int by, int bz, float threshold, int wtype, int encoder);
std::string header_text_sub(int bx, int by, int bz, int sbx, int sby, int sbz, float threshold, int wtype,
                            int encoder);
// size_t header offset + binary-ocean title: where the payloads start
long long mini_header_bytes();
// payload may already sit at out + mini_header_bytes() (no copy then)
long long image_bytes(long long payload, int nchunks, long long nblocks, const std::string &header);
long long write_image(uint8_t *out, const uint8_t *payload, long long payload_bytes, const long long *chunk_off,
                      int nchunks, const int *block_chunk, const int *block_subid, int bx, int by, int bz,
                      const std::string &header);

// several ranks writing one file: rank parts, mini header, tail
long long write_part(uint8_t *out, const uint8_t *payload, long long payload_bytes, const long long *chunk_off,
                     int nchunks);
void write_mini(uint8_t *out, long long header_offset);
long long tail_bytes(long long nblocks, int nranks, const std::string &header);
long long write_tail(uint8_t *out, const std::string &header, int bx, int by, int bz, int nranks, int bpc,
                     const long long *part_bytes, const int *part_chunks);

struct Parsed {
    int bx = 0, by = 0, bz = 0;
    int encoder = -1;  // 0 none, 1 lz4, 2 zlib
    float threshold = 0.f;
    std::string wavelets;
    std::vector<long long> chunk_start, chunk_size;  // absolute file offsets / sizes
    std::vector<int> block_chunk, block_subid;       // per block in grid order
    int max_subid = 0;
};
int parse_image(const uint8_t *img, long long size, Parsed &out, std::string &err);

}  // namespace czf
