// cz_layout.cuh -- index maps between the kernels' block layout and the
// reference's positional layout.
//
// The reference transforms a block with in-place positional transposes that
// are never undone (WaveletsOnInterval.h:240-276; "we don't need this" at
// :246,265), so a coefficient's position in the final array depends on the
// level that produced it. The kernels instead keep every coefficient at its
// mathematical index: physical (x,y,z) holds the coefficient with index x
// along the field's x axis, y along y and z along z, and the 1D sweeps run
// along the mathematical axes in the order the reference applies them:
//
//   level 32: x, y, z        final position [y][x][z]
//   level 16: z, x, y        final position [x][z][y]   (on the [0,16)^3 corner)
//   level  8: y, z, x        final position [z][y][x]   (on the [0,8)^3 corner)
//   coarse 4^3 untouched     position [z][y][x]
//
// (derived from sweep3D applied to the positional array each level hands to
// the next, FullWaveletTransform.h:44-56). Thresholding then visits the
// coefficients in the reference's order (FullWaveletTransform.h:58-96) through
// these maps; the mask index is the positional index x + 32*(y + 32*z)
// (:86) and the survivor stream is coarse-first, then per level 8, 16, 32
// the octant codes 1..7 in z,y,x order (:63-93, base :162-176).
#pragma once
#include "cz_arith.cuh"

namespace cz {

CZ_HD int imax3(int a, int b, int c)
{
    const int m = a > b ? a : b;
    return m > c ? m : c;
}

// Positional (mask) index of the coefficient stored at physical (x,y,z).
CZ_HD int mask_index(int x, int y, int z)
{
    const int m = imax3(x, y, z);
    if (m >= 16) return z + 32 * (x + 32 * y);
    if (m >= 8) return y + 32 * (z + 32 * x);
    return x + 32 * (y + 32 * z);
}

// Physical (x,y,z) of positional index p.
CZ_HD void phys_of_pos(int px, int py, int pz, int &x, int &y, int &z)
{
    const int m = imax3(px, py, pz);
    if (m >= 16) {
        x = py; y = pz; z = px;
    } else if (m >= 8) {
        x = pz; y = px; z = py;
    } else {
        x = px; y = py; z = pz;
    }
}

// Positional coordinates of the s-th entry of the survivor stream order.
CZ_HD void pos_of_stream(int s, int &px, int &py, int &pz)
{
    if (s < 64) {
        px = s & 3; py = (s >> 2) & 3; pz = s >> 4;
        return;
    }
    int lh, base;  // log2 of the half size, stream offset of the level
    if (s < 512) { lh = 2; base = 64; }
    else if (s < 4096) { lh = 3; base = 512; }
    else { lh = 4; base = 4096; }
    const int r = s - base;
    const int code = (r >> (3 * lh)) + 1;
    const int w = r & ((1 << (3 * lh)) - 1);
    const int hh = 1 << lh;
    px = hh * (code & 1) + (w & (hh - 1));
    py = hh * ((code >> 1) & 1) + ((w >> lh) & (hh - 1));
    pz = hh * ((code >> 2) & 1) + (w >> (2 * lh));
}

// Stream index of positional (px,py,pz): inverse of pos_of_stream.
CZ_HD int stream_of_pos(int px, int py, int pz)
{
    const int m = imax3(px, py, pz);
    if (m < 4) return px + 4 * (py + 4 * pz);
    const int lh = m >= 16 ? 4 : (m >= 8 ? 3 : 2);
    const int base = m >= 16 ? 4096 : (m >= 8 ? 512 : 64);
    const int hh = 1 << lh;
    const int code = (px >> lh) | ((py >> lh) << 1) | ((pz >> lh) << 2);
    const int w = (px & (hh - 1)) | ((py & (hh - 1)) << lh) | ((pz & (hh - 1)) << (2 * lh));
    return base + ((code - 1) << (3 * lh)) + w;
}

}  // namespace cz
