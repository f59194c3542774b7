"""The .cz parser behind cz_image_info and cz_decompress_image (host code,
cz_format.cpp) on damaged files: a valid image built from the oracle's LZ4
chunks by the host writer, then bytes of its mini header, ASCII header,
block metadata and LUTs changed, files cut short, and block counts, chunk
counts and LUT offsets set to values whose products or sums overflow. Every
case parses or returns an error code; none crashes the process."""
import ctypes as C
import re

import numpy as np
import pytest

from oracle import czoracle as O

CZ_OK, CZ_E_ARG, CZ_E_CORRUPT = 0, -1, -3


@pytest.fixture(scope="module")
def lib():
    from cubismz_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="module")
def image(lib, small_field, tmp_path_factory):
    from cubismz_gb300 import api, shard
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    payload, off = O.field_compress(small_field, eps, 1, 4, 1, 1, 1)
    part, n = shard.part_from_host(payload, off)
    path = str(tmp_path_factory.mktemp("cz") / "field.cz")
    shard.write_file(path, part, n, small_field.shape, api.params(eps, 1, 4, True, "lz4", 1))
    with open(path, "rb") as f:
        return f.read(), n


def info(lib, img):
    buf = np.frombuffer(bytes(img), np.uint8).copy() if len(img) else np.zeros(1, np.uint8)
    dims = (C.c_int * 3)()
    enc = C.c_int(-9)
    rc = lib.cz_image_info(C.c_void_p(buf.ctypes.data), len(img), dims, C.byref(enc))
    return rc, (dims[0], dims[1], dims[2]), enc.value


def test_valid_image_parses(lib, image, small_field):
    img, _ = image
    rc, dims, enc = info(lib, img)
    nz, ny, nx = small_field.shape
    assert rc == CZ_OK and dims == (nx, ny, nz) and enc == 1


def test_changed_bytes_and_cuts(lib, image):
    img, _ = image
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    rng = np.random.default_rng(4)
    regions = [(0, 8), (8, 60), (hoff, len(img)), (len(img) - 12, len(img)), (hoff - 64, hoff)]
    for _ in range(1500):
        lo, hi = regions[int(rng.integers(0, len(regions)))]
        b = bytearray(img)
        for _ in range(int(rng.integers(1, 4))):
            b[int(rng.integers(lo, hi))] = int(rng.integers(0, 256))
        rc, _, _ = info(lib, b)
        assert rc in (CZ_OK, CZ_E_ARG, CZ_E_CORRUPT)
    for cut in sorted(set(int(x) for x in rng.integers(0, len(img), 200))):
        rc, _, _ = info(lib, img[:cut])
        assert rc in (CZ_E_ARG, CZ_E_CORRUPT)


def _sub(img, key, value):
    """The image with the ASCII header line `key: ...` replaced."""
    pat = re.compile(rb"\n" + key.encode() + rb":[^\n]*\n")
    assert pat.search(img)
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    new = pat.sub(b"\n" + key.encode() + b": " + value.encode() + b"\n", img[hoff:], count=1)
    return img[:hoff] + new


@pytest.mark.parametrize("key,value", [
    ("Blocks", "2000000000 x 2000000000 x 2000000000"),
    ("Blocks", "65536 x 65536 x 65536"),
    ("Blocks", "2147483647 x 1 x 1"),
    ("Blocks", "-4 x 2 x 2"),
    ("SubdomainBlocks", "2147483647 x 2147483647 x 2147483647"),
    ("SubdomainBlocks", "1 x 1 x 0"),
    ("SubdomainBlocks", "3 x 5 x 7"),
])
def test_overflowing_block_counts_are_rejected(lib, image, key, value):
    img, _ = image
    rc, _, _ = info(lib, _sub(img, key, value))
    assert rc in (CZ_E_ARG, CZ_E_CORRUPT)


@pytest.mark.parametrize("agg,nch", [(2 ** 63 - 1, 1), (2 ** 64 - 1, 1), (2 ** 63 + 8, 2), (16, 2 ** 31 - 1),
                                     (0, 1), (None, -1), (None, 0)])
def test_overflowing_header_lut_is_rejected(lib, image, agg, nch):
    img, n = image
    b = bytearray(img)
    if agg is not None:
        b[-12:-4] = np.uint64(agg).tobytes()
    b[-4:] = np.int32(nch).tobytes()
    rc, _, _ = info(lib, b)
    assert rc in (CZ_E_ARG, CZ_E_CORRUPT)


@pytest.mark.parametrize("k,value", [(0, 2 ** 63 + 5), (0, 2 ** 64 - 1), (1, 0), (-1, 2 ** 62), (-1, 2 ** 64 - 8)])
def test_out_of_range_chunk_offsets_are_rejected(lib, image, k, value):
    img, n = image
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    b = bytearray(img)
    lut0 = hoff - 8 * n  # the rank's chunk offsets end at the header
    i = k % n
    b[lut0 + 8 * i:lut0 + 8 * i + 8] = np.uint64(value).tobytes()
    rc, _, _ = info(lib, b)
    assert rc in (CZ_E_ARG, CZ_E_CORRUPT)


@pytest.mark.gpu
def test_damaged_chunks_decode_or_fail_cleanly(gpu_lib, image, small_field):
    """cz_decompress_image on images with changed chunk bytes: each decodes
    or raises CzError, and afterwards the intact image still decodes to the
    same field (the context stays usable)."""
    import cubismz_gb300 as cz
    img, n = image
    good = cz.decompress_image(img, 1, True)
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    mini = 8 + len(b"\n==============START-BINARY-OCEAN==============\n")
    rng = np.random.default_rng(9)
    failed = 0
    for _ in range(60):
        b = bytearray(img)
        for _ in range(int(rng.integers(1, 4))):
            b[int(rng.integers(mini, hoff - 8 * n))] = int(rng.integers(0, 256))
        try:
            cz.decompress_image(bytes(b), 1, True)
        except cz.CzError:
            failed += 1
    assert failed > 0
    assert np.array_equal(cz.decompress_image(img, 1, True).view(np.uint32), good.view(np.uint32))



@pytest.mark.parametrize("subid", [64, 10 ** 6, 2 ** 31 - 1])
def test_large_record_index_is_rejected(lib, image, subid):
    """A block whose metadata names a record index (subid) beyond the blocks
    of its subdomain is damage: refused before any decode buffer is sized
    by it (the 128^3 field has 64 blocks in one subdomain)."""
    img, _ = image
    marker = b"==============START-BINARY-METABLOCKS==============\n"
    m0 = img.index(marker) + len(marker)
    b = bytearray(img)
    b[m0 + 4:m0 + 8] = np.int32(subid).tobytes()  # BlockMetadata {chunk, subid, ix, iy, iz} of block 0
    rc, _, _ = info(lib, b)
    assert rc == CZ_E_CORRUPT
    b[m0 + 4:m0 + 8] = np.int32(63).tobytes()  # in range: parses (the block's bytes are simply elsewhere)
    rc, _, _ = info(lib, b)
    assert rc == CZ_OK
