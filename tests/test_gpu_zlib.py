"""zlib streams on the GPU: every DEFLATE block type decodes like zlib
itself, malformed input is rejected, and the published golden file (demo.h5,
wtype 3, threshold 5e-5, Encoder: zlib, 15 records per chunk) decodes on the
GPU to the published RES line."""
import os
import tempfile
import zlib

import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import zlib_chunks
from tests.test_res import stats_f64

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


def _samples(small_field):
    rng = np.random.default_rng(3)
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    return [b"", b"a", bytes(70000), rng.integers(0, 256, 50000, np.uint8).tobytes(),
            b"abcabcabd" * 3000, rng.integers(0, 5, 120000, np.uint8).tobytes(),
            bytes(raw[off[0]:off[15]]), bytes(raw[off[20]:off[21]])]


def test_inflate_matches_zlib(cz, small_field):
    for d in _samples(small_field):
        for level in (0, 1, 6, 9):
            for strategy in (zlib.Z_DEFAULT_STRATEGY, zlib.Z_FIXED, zlib.Z_FILTERED):
                co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
                z = co.compress(d) + co.flush()
                assert cz.zlib_decompress(z, len(d)) == d


def test_inflate_rejects_malformed(cz):
    rng = np.random.default_rng(7)
    d = rng.integers(0, 8, 30000, np.uint8).tobytes()
    z = zlib.compress(d, 6)
    bad = [z[:len(z) // 2], z[:-1], z[:-4] + bytes(4), bytes([0x78, 0x9c, 0xff]) + z[3:], b"\x00\x00", z[2:]]
    for b in bad:
        with pytest.raises(cz.CzError):
            cz.zlib_decompress(b, len(d))
    with pytest.raises(cz.CzError):
        cz.zlib_decompress(z, len(d) - 1)  # output capacity
    for _ in range(40):
        junk = bytes([0x78, 0x9c]) + rng.integers(0, 256, int(rng.integers(1, 400)), np.uint8).tobytes()
        try:
            want = zlib.decompress(junk)
        except zlib.error:
            want = None
        if want is None or len(want) > 65536:
            with pytest.raises(cz.CzError):
                cz.zlib_decompress(junk, 65536)
        else:
            assert cz.zlib_decompress(junk, 65536) == want


def test_published_golden_zlib_file_on_gpu(cz, golden, demo_field):
    from cubismz_gb300 import api, shard
    raw, off = O.field_compress(demo_field, 5e-5, 3, 0, 0, 0, 1)
    z = zlib_chunks(raw, off, 15, 64)
    offs = np.concatenate([[0], np.cumsum([len(c) for c in z])]).astype(np.int64)
    part, n = shard.part_from_host(np.frombuffer(b"".join(z), np.uint8), offs)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "demo.cz")
        size = shard.write_file(path, part, n, demo_field.shape, api.params(5e-5, 3, 0, False, "zlib", 15))
        img = open(path, "rb").read()
    assert size == len(img) == golden["reference_rebuilt_cz_bytes"]
    dec = cz.decompress_image(img, 3, False)
    assert np.array_equal(dec, O.field_decompress(raw, off, demo_field.shape, 3))
    assert cz.res_line(stats_f64(demo_field, dec), size) == golden["published_res"]
