"""GPU-written .cz files read by the reference's own reader.

tests/golden/gpu_small_{lz4,zlib}.cz were written on a GB300 by
cz_compress_to_image (tests/golden/make_gpu_images.py: the 128^3 field of
the plain-method workload, threshold 1e-2 of its range, wtype 1, zero-bits
4, shuffle). The reference's reader (load_file + load_block2,
Reader_WaveletCompression.h:255-560, 635-754), compiled from the reference
sources into oracle/_ref with the matching zero-bits/shuffle/encoder
options, must decode them to exactly the field the oracle decodes from its
own records of the same input. Runs where the reference tree was built
(CPU); skipped elsewhere."""
import os
import tempfile

import numpy as np
import pytest

from oracle import czoracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def one_rank_chunks(img):
    """Chunk payloads of a one-rank image: the part starts after the mini
    header; the rank's LUT of chunk offsets (relative to the part) ends at
    the ASCII header; the HeaderLUT's last 4 bytes give the chunk count
    (SerializerIO_WaveletCompression_MPI_Simple.h:371-466)."""
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    n = int(np.frombuffer(img[-4:], np.int32)[0])
    mini = 8 + len(b"\n==============START-BINARY-OCEAN==============\n")
    lut = [int(x) for x in np.frombuffer(img[hoff - 8 * n:hoff], np.uint64)] + [hoff - 8 * n - mini]
    return [img[mini + lut[c]:mini + lut[c + 1]] for c in range(n)]


@pytest.fixture(scope="module")
def expected():
    import sys
    sys.path.insert(0, GOLDEN)
    from make_gpu_images import REL_THR, SHUFFLE, WTYPE, ZEROBITS, field_and_eps
    field, eps = field_and_eps()
    raw, roff = O.field_compress(field, eps, WTYPE, ZEROBITS, int(SHUFFLE), 0, 1)
    return field, eps, O.field_decompress(raw, roff, field.shape, WTYPE, int(SHUFFLE)), (WTYPE, ZEROBITS, SHUFFLE)


@pytest.mark.parametrize("enc", ["lz4", "zlib"])
def test_reference_reader_decodes_gpu_image(expected, enc):
    field, eps, want, (wtype, zb, sh) = expected
    L = O.ref(zb, sh, enc)
    if L is None:
        pytest.skip("the reference build (oracle/_ref) is not available here")
    path = os.path.join(GOLDEN, f"gpu_small_{enc}.cz")
    got = O.ref_read_cz(L, path, wtype)
    assert got.shape == field.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("enc", ["lz4", "zlib"])
def test_gpu_image_header_and_chunks(expected, enc):
    """The image's header names the encoder and the grid, and its chunks
    decode (restated reference decoders) to the oracle's records."""
    import zlib
    field, eps, _, (wtype, zb, sh) = expected
    with open(os.path.join(GOLDEN, f"gpu_small_{enc}.cz"), "rb") as f:
        img = f.read()
    text = img[int(np.frombuffer(img[:8], np.uint64)[0]):]
    assert f"Encoder: {enc}".encode() in text and b"Blocks: 4 x 4 x 4" in text
    raw, roff = O.field_compress(field, eps, wtype, zb, int(sh), 0, 1)
    chunks = one_rank_chunks(img)
    assert len(chunks) == 64
    for c, ch in enumerate(chunks):
        want = raw[roff[c]:roff[c + 1]]
        if enc == "lz4":
            n, out = O.lz4_decompress(np.frombuffer(ch, np.uint8), len(want))
            assert n == len(want) and np.array_equal(out, want)
        else:
            assert zlib.decompress(ch) == want.tobytes()
