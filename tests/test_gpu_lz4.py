"""GPU LZ4 stage: reference-encoded streams decode with the GPU decoder;
GPU-encoded streams decode with the restated reference decoder (and the
reference's own, where it was built); malformed input is rejected without
faulting."""
import os

import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import sha

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


def test_gpu_decodes_reference_lz4(cz, golden):
    data = open(os.path.join(os.path.dirname(__file__), "golden", "ref_lz4_chunks.bin"), "rb").read()
    pos = 0
    for entry in golden["ref_lz4_chunks"]:
        zn, rn = np.frombuffer(data[pos:pos + 8], np.int32)
        z = data[pos + 8:pos + 8 + zn]
        pos += 8 + zn
        out = cz.lz4_decompress(z, int(rn))
        assert len(out) == entry["raw_bytes"] and sha(out) == entry["raw_sha256"]


def test_gpu_lz4_roundtrip(cz, small_field):
    rng = np.random.default_rng(9)
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    samples = [b"", b"x", bytes(12), bytes(13), bytes(70000), rng.integers(0, 256, 100000, np.uint8).tobytes(),
               (b"0123456789abcdef" * 5000), bytes(raw[off[0]:off[1]]), bytes(raw[off[7]:off[9]])]
    # short repeats over a small alphabet at every distance (window and
    # super-window boundaries), and long runs crossing them
    toks = [rng.integers(0, 8, 7, np.uint8).tobytes() for _ in range(40)]
    samples.append(b"".join(toks[i] for i in rng.integers(0, 40, 30000)))
    samples.append(bytes(3000) + rng.integers(0, 256, 2500, np.uint8).tobytes() + bytes(9000) + b"\x01" * 70000)
    # period 2^18: hash-table positions are kept modulo 2^18, so entries one
    # period back alias to offset 0 and must be rejected
    blk = rng.integers(0, 4, 1 << 18, np.uint8).tobytes()
    samples.append(blk + blk)
    L = O.ref(4, 1, "lz4")
    for d in samples:
        z = cz.lz4_compress(d)
        assert len(z) <= len(d) + len(d) // 255 + 16
        n, out = O.lz4_decompress(z, len(d))
        assert n == len(d) and out.tobytes() == d
        assert cz.lz4_decompress(z, len(d)) == d
        if L is not None:
            n2, out2 = O.ref_lz4_decompress(L, z, len(d))
            assert n2 == len(d) and out2.tobytes() == d


def test_gpu_lz4_rejects_malformed(cz):
    d = bytes(4000) + b"pattern!" * 500
    z = cz.lz4_compress(d)
    with pytest.raises(cz.CzError):
        cz.lz4_decompress(z, 100)  # output too small
    bad = bytearray(z)
    bad[0] = 0xF0  # literal length runs past the input
    with pytest.raises(cz.CzError):
        cz.lz4_decompress(bytes(bad[:3]), len(d))
    rng = np.random.default_rng(1)
    for _ in range(20):
        junk = rng.integers(0, 256, int(rng.integers(1, 300)), np.uint8).tobytes()
        try:
            out = cz.lz4_decompress(junk, 4096)
            n, ref = O.lz4_decompress(junk, 4096)
            assert n == len(out) and ref.tobytes() == out
        except cz.CzError:
            n, _ = O.lz4_decompress(junk, 4096)
            assert n <= 0


def test_gpu_lz4_decodes_constructed_streams(cz):
    """Valid streams with overlapping copies, every offset class and long
    length fields decode as the restated reference decoder decodes them;
    with one byte less of output capacity both reject them."""
    from tests.helpers import lz4_random_stream
    rng = np.random.default_rng(21)
    for t in range(40):
        z, ref = lz4_random_stream(rng, int(rng.integers(1, 400)))
        n, o = O.lz4_decompress(z, len(ref))
        assert n == len(ref) and o.tobytes() == ref  # the construction is valid
        assert cz.lz4_decompress(z, len(ref)) == ref
        assert cz.lz4_decompress(z, len(ref) + 100) == ref
        for cap in (len(ref) - 1, len(ref) // 2):
            n, _ = O.lz4_decompress(z, cap)
            assert n <= 0
            with pytest.raises(cz.CzError):
                cz.lz4_decompress(z, cap)


def test_gpu_lz4_returns_the_reference_decoder_results(cz):
    """Through the C ABI, cz_lz4_decompress writes what the reference's
    LZ4_uncompress_unknownOutputSize returned on the same input and
    capacity -- the output size, or minus the input position of the error --
    and the same output bytes."""
    import ctypes as C
    import hashlib
    from tests.helpers import lz4_cases
    ctx = cz.context(0)
    for data, cap, ref, ref_sha in lz4_cases():
        src = np.frombuffer(data, np.uint8).copy()
        dst = np.zeros(max(cap, 1), np.uint8)
        n = C.c_int(0)
        rc = ctx.L.cz_lz4_decompress(ctx.h, src.ctypes.data_as(C.POINTER(C.c_uint8)), src.size,
                                     dst.ctypes.data_as(C.POINTER(C.c_uint8)), cap, C.byref(n))
        assert n.value == ref, (len(data), cap, n.value, ref)
        assert (rc == 0) == (ref >= 0)
        if ref > 0:
            assert hashlib.sha256(dst[:ref].tobytes()).hexdigest() == ref_sha



def test_gpu_lz4_effort_levels(cz, small_field):
    """Every parse effort writes streams that the restated reference decoder
    and the GPU decoder read back exactly, on the round-trip samples and on
    a field's record chunks (also through the image writer's pipelined path
    and the zlib stage's LZ77 parse); on the record chunks a higher effort
    never writes more bytes."""
    import torch
    rng = np.random.default_rng(5)
    raw, roff = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    toks = [rng.integers(0, 8, 7, np.uint8).tobytes() for _ in range(40)]
    samples = [b"", bytes(13), rng.integers(0, 256, 5000, np.uint8).tobytes(), b"ab" * 3000 + b"abc" * 2000,
               b"".join(toks[i] for i in rng.integers(0, 40, 20000)), bytes(raw[roff[3]:roff[4]])]
    ref_field = O.field_decompress(raw, roff, small_field.shape, 1, 1)
    f = torch.from_numpy(small_field).cuda()
    ctx = cz.context(0)
    sizes = []
    try:
        for effort in (0, 1, 2):
            ctx.set_lz4_effort(effort)
            for d in samples:
                z = cz.lz4_compress(d)
                n, out = O.lz4_decompress(z, len(d))
                assert n == len(d) and out.tobytes() == d
                assert cz.lz4_decompress(z, len(d)) == d
            cf = cz.compress_field(f, 1e-3, 1, 4, True, encoder="lz4")
            data, off = cf.to_device()
            o, dd = off.cpu().numpy(), data.cpu().numpy()
            for c in range(len(o) - 1):
                n, out = O.lz4_decompress(dd[o[c]:o[c + 1]], int(roff[c + 1] - roff[c]))
                assert n == roff[c + 1] - roff[c] and np.array_equal(out, raw[roff[c]:roff[c + 1]])
            sizes.append(int(o[-1]))
            dec = cz.decompress_field(data, off, small_field.shape, 1, True, encoder="lz4").cpu().numpy()
            assert np.array_equal(dec, ref_field)
            img = cz.compress_to_image(small_field, 1e-3, 1, 4, True, encoder="lz4")
            assert np.array_equal(cz.decompress_image(img, 1, True), ref_field)
            cz_ = cz.compress_field(f, 1e-3, 1, 4, True, encoder="zlib")
            zd, zo = cz_.to_device()
            dec = cz.decompress_field(zd, zo, small_field.shape, 1, True, encoder="zlib").cpu().numpy()
            assert np.array_equal(dec, ref_field)
        with pytest.raises(cz.CzError):
            ctx.set_lz4_effort(3)
    finally:
        ctx.set_lz4_effort(1)
    assert sizes[1] <= sizes[0] and sizes[2] <= sizes[1], sizes
