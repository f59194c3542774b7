"""zlib streams on the GPU: every DEFLATE block type decodes like zlib
itself, malformed input is rejected, and the published golden file (demo.h5,
wtype 3, threshold 5e-5, Encoder: zlib, 15 records per chunk) decodes on the
GPU to the published RES line. Streams written by the GPU encoder decode
with zlib to their input; fields and .cz files written with Encoder: zlib
hold the oracle's records and decode bit-exactly."""
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


def test_inflate_edited_streams_like_zlib(cz):
    """Valid streams (dynamic, fixed and stored blocks) with one byte
    changed: the GPU inflate fails where zlib fails and otherwise returns
    zlib's bytes."""
    rng = np.random.default_rng(11)
    d = (rng.integers(0, 6, 20000, np.uint8).tobytes() + bytes(3000) + b"pattern-" * 400
         + rng.integers(0, 256, 2000, np.uint8).tobytes())
    streams = [zlib.compress(d, 6), zlib.compress(d, 1), zlib.compress(d, 0)]
    co = zlib.compressobj(9, zlib.DEFLATED, 15, 9, zlib.Z_FIXED)
    streams.append(co.compress(d) + co.flush())
    for z in streams:
        for _ in range(25):
            e = bytearray(z)
            pos = int(rng.integers(0, len(z)))
            e[pos] = (e[pos] + int(rng.integers(1, 256))) & 255
            e = bytes(e)
            try:
                want = zlib.decompress(e)
            except zlib.error:
                want = None
            if want is None or len(want) > len(d):
                with pytest.raises(cz.CzError):
                    cz.zlib_decompress(e, len(d))
            else:
                assert cz.zlib_decompress(e, len(d)) == want


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


def _encode_samples(small_field):
    rng = np.random.default_rng(11)
    unit = rng.integers(0, 256, 32768, np.uint8).tobytes()
    return _samples(small_field) + [
        b"ab", bytes(259), bytes(260), bytes(261), bytes(517), bytes(300000),
        rng.integers(0, 256, 300000, np.uint8).tobytes(), unit + unit[:5000] + unit[:300],
        bytes(rng.integers(0, 3, 100000, np.uint8)) * 2, (b"\x00" * 1000 + b"\x01" * 7) * 300]


def test_deflate_streams_decode_with_zlib(cz, small_field):
    """cz.zlib_compress: zlib and the GPU inflate read every stream back;
    sizes stay within the stored bound."""
    for d in _encode_samples(small_field):
        z = cz.zlib_compress(d)
        assert z[:2] == b"\x78\x9c"
        assert zlib.decompress(z) == d, len(d)
        assert cz.zlib_decompress(z, len(d)) == d
        assert len(z) <= len(d) + 6 * (len(d) // 1024 + 2) + 8


def test_deflate_ratio_against_zlib_default(cz, small_field):
    """Field chunks of shuffled records (a DEFLATE block per mask and byte
    plane) come out no larger than zlib at the reference's
    Z_DEFAULT_COMPRESSION on the same records (2 % slack for the parse);
    generic input within 15 %."""
    import torch
    f = torch.from_numpy(small_field).cuda()
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="zlib")
    ref = sum(len(zlib.compress(bytes(raw[roff[i]:roff[i + 1]]), 6)) for i in range(len(roff) - 1))
    assert cf.nbytes <= 1.02 * ref, (cf.nbytes, ref)
    gpu = sum(len(cz.zlib_compress(bytes(raw[roff[i]:roff[i + 1]]))) for i in range(0, len(roff) - 1, 9))
    ref = sum(len(zlib.compress(bytes(raw[roff[i]:roff[i + 1]]), 6)) for i in range(0, len(roff) - 1, 9))
    assert gpu <= 1.15 * ref, (gpu, ref)


@pytest.mark.parametrize("bpc", [1, 15])
def test_field_with_zlib_encoder(cz, small_field, bpc):
    """compress_field(encoder="zlib"): every chunk inflates (with zlib) to
    the oracle's records, and the field decodes bit-exactly on the GPU."""
    import torch
    f = torch.from_numpy(small_field).cuda()
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="zlib", blocks_per_chunk=bpc)
    data, off = cf.to_device()
    h, o = data.cpu().numpy().tobytes(), off.cpu().numpy()
    nb = len(roff) - 1
    for c in range(len(o) - 1):
        b0, b1 = c * bpc, min(nb, (c + 1) * bpc)
        want = bytes(raw[roff[b0]:roff[b1]])
        assert zlib.decompress(h[o[c]:o[c + 1]]) == want, c
    dec = cz.decompress_field(data, off, small_field.shape, 1, True, encoder="zlib", blocks_per_chunk=bpc)
    assert np.array_equal(dec.cpu().numpy(), O.field_decompress(raw, roff, small_field.shape, 1, 1))


def test_zlib_cz_image(cz, small_field):
    """A .cz image with Encoder: zlib from the GPU: header names the
    encoder, every chunk inflates with zlib to the oracle's record, and the
    image decodes on the GPU bit-exactly."""
    from tests.helpers import parse_cz
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    img = cz.compress_to_image(small_field, eps, 1, 4, True, encoder="zlib")
    info = parse_cz(bytes(img))
    assert info["keys"]["Encoder"] == "zlib"
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    chunks = [c for r in info["ranks"] for c in r]
    assert len(chunks) == len(roff) - 1
    for i, c in enumerate(chunks):
        assert zlib.decompress(c) == bytes(raw[roff[i]:roff[i + 1]])
    dec = cz.decompress_image(img, 1, True)
    assert np.array_equal(dec, O.field_decompress(raw, roff, small_field.shape, 1, 1))
    L = O.ref(4, 1, "zlib")
    if L is not None:  # the reference reader decodes the GPU-written file
        with tempfile.NamedTemporaryFile(suffix=".cz") as t:
            t.write(bytes(img))
            t.flush()
            assert np.array_equal(O.ref_read_cz(L, t.name, 1), dec)
