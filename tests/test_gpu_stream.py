"""GPU field pipeline with the LZ4 stage and .cz images: bit-exact round
trips at the small size, size-independent properties at the 512^3 size."""
import numpy as np
import pytest

from oracle import czoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


def test_lz4_field_roundtrip(cz, small_field):
    import torch
    f = torch.from_numpy(small_field).cuda()
    cf = cz.compress_field(f, 1e-3, 1, 4, True, encoder="lz4")
    data, off = cf.to_device()
    o = off.cpu().numpy()
    d = data.cpu().numpy()
    raw, roff = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    assert cf.raw_bytes == int(roff[-1])
    for c in range(len(o) - 1):
        n, out = O.lz4_decompress(d[o[c]:o[c + 1]], int(roff[c + 1] - roff[c]))
        assert n == roff[c + 1] - roff[c] and np.array_equal(out, raw[roff[c]:roff[c + 1]])
    dec = cz.decompress_field(data, off, small_field.shape, 1, True, encoder="lz4").cpu().numpy()
    assert np.array_equal(dec, O.field_decompress(raw, roff, small_field.shape, 1, 1))


def test_cz_image_roundtrip(cz, small_field):
    img = cz.compress_to_image(small_field, 1e-3, 1, 4, True, encoder="lz4")
    shape, enc = cz.image_info(img)
    assert shape == small_field.shape and enc == 1
    dec = cz.decompress_image(img, 1, True)
    raw, roff = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    assert np.array_equal(dec, O.field_decompress(raw, roff, small_field.shape, 1, 1))
    L = O.ref(4, 1, "lz4")
    if L is not None:  # the reference reader decodes the GPU-written file
        import tempfile
        with tempfile.NamedTemporaryFile(suffix=".cz") as t:
            t.write(bytes(img))
            t.flush()
            assert np.array_equal(O.ref_read_cz(L, t.name, 1), dec)


@pytest.mark.parametrize("world", [2, 4])
def test_multi_rank_image_on_gpu(cz, small_field, world):
    """A .cz image as 2 or 4 ranks write it (each rank's chunks, then its
    LUT, then the next rank's part) decodes on the GPU to the oracle's
    field: the reader packs the ranks' chunks before one launch."""
    from tests.helpers import multi_rank_image
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    dec = cz.decompress_image(multi_rank_image(small_field, eps, world), 1, True)
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    want = O.field_decompress(raw, roff, small_field.shape, 1, 1)
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))


def test_large_field_properties(cz):
    """512^3 (4096 blocks): per-block records equal the oracle on a sample of
    blocks, the LZ4 stage round-trips every chunk, and decompression equals
    the oracle's decode of the same records."""
    import torch
    from cubismz_gb300 import synth
    field = synth.config_field("large", 0)
    rng_thr = 1e-3 * float(field.max() - field.min())
    f = torch.from_numpy(field).cuda()
    cf = cz.compress_field(f, rng_thr, 1, 4, True, encoder="lz4")
    data, off = cf.to_device()
    dec = cz.decompress_field(data, off, field.shape, 1, True, encoder="lz4")
    cf_raw = cz.compress_field(f, rng_thr, 1, 4, True, encoder="none")
    rdata, roff = cf_raw.to_device()
    rd, ro = rdata.cpu().numpy(), roff.cpu().numpy()
    rng = np.random.default_rng(0)
    for g in rng.choice(4096, 48, replace=False):
        bz, by, bx = g // 256, (g // 16) % 16, g % 16
        blk = field[bz * 32:bz * 32 + 32, by * 32:by * 32 + 32, bx * 32:bx * 32 + 32]
        want = O.block_compress(blk, np.float32(rng_thr), 1, 4, 1)
        assert np.array_equal(rd[ro[g] + 4:ro[g + 1]], want)
    full = O.field_decompress(rd, ro, field.shape, 1, 1, 0, 1, 0)
    assert np.array_equal(dec.cpu().numpy(), full)
    assert np.isfinite(full).all()


def test_fused_decode_and_error_norms(cz, small_field):
    """diff_field decodes and computes cz2diff's statistics in one pass:
    maxima and range exact, sums to 1e-12 of binary64, same RES line."""
    import torch
    from tests.test_res import stats_f64
    f = torch.from_numpy(small_field).cuda()
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="lz4")
    data, off = cf.to_device()
    out = torch.empty_like(f)
    got = cz.diff_field(data, off, small_field.shape, f, 1, True, encoder="lz4", file_bytes=cf.nbytes, out=out)
    dec = out.cpu().numpy()
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    assert np.array_equal(dec, O.field_decompress(raw, roff, small_field.shape, 1, 1))
    want = stats_f64(small_field, dec)
    for k in ("e_inf", "n_inf", "min", "max", "n"):
        assert got[k] == want[k], k
    for k in ("e_1", "n_1", "e_2", "n_2"):
        assert abs(got[k] - want[k]) <= 1e-12 * abs(want[k]), k
    assert got["res_line"] == cz.res_line(want, cf.nbytes)


@pytest.mark.parametrize("encoder", ["lz4", "zlib"])
def test_all_coefficients_kept(cz, small_field, encoder):
    """A negative threshold keeps every coefficient: records of the maximum
    size (4 + 4096 + 4*32768 bytes) with byte planes close to
    incompressible. Both lossless stages round-trip them through the field
    and the pipelined image paths, bit-exactly to the oracle."""
    import torch
    field = np.ascontiguousarray(small_field[:64])
    raw, roff = O.field_compress(field, -1.0, 1, 0, 1, 0, 1)
    assert set(np.diff(roff).tolist()) == {4 + 4096 + 4 * 32768}
    want = O.field_decompress(raw, roff, field.shape, 1, 1)
    cf = cz.compress_field(torch.from_numpy(field).cuda(), -1.0, 1, 0, True, encoder=encoder)
    data, off = cf.to_device()
    dec = cz.decompress_field(data, off, field.shape, 1, True, encoder=encoder).cpu().numpy()
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))
    img = cz.compress_to_image(field, -1.0, 1, 0, True, encoder=encoder)
    assert np.array_equal(cz.decompress_image(img, 1, True).view(np.uint32), want.view(np.uint32))


def test_lz4_planes_left_in_the_input(cz):
    """A one-record chunk whose byte planes 1 and 2 sit in one literal run:
    the LZ4 decoder leaves them in its input and the decode kernel reads
    them there; the match right after the run and a later one copy from
    planes 2 and 1, so they read the input too. The decoded block equals
    the oracle's decode of the record."""
    import torch
    from tests.helpers import _lz4_len
    rng = np.random.default_rng(3)
    block = rng.standard_normal((32, 32, 32)).astype(np.float32)
    rec = O.block_compress(block, 0.5, 1, 4, 1)
    S = (len(rec) - 4096) // 4
    assert S >= 600
    chunk = bytearray(np.int32(len(rec)).tobytes()) + bytearray(rec.tobytes())
    P1, P2, P3 = 4 + 4096 + S, 4 + 4096 + 2 * S, 4 + 4096 + 3 * S
    for a in (P1, P2, P3, P3 + 12):  # benign bytes: mantissa bits, or an exponent near 1
        chunk[a:a + 8] = b"\x3f" * 8
    seen, x, y = {}, None, None
    for i in range(4, P1 - 8):
        k = bytes(chunk[i:i + 4])
        if k in seen:
            x, y = i, seen[k]
            break
        seen.setdefault(k, i)
    assert x is not None
    z = bytearray()

    def seq(lits, off, ml):
        z.append((min(len(lits), 15) << 4) | min(ml - 4, 15))
        if len(lits) >= 15:
            _lz4_len(z, len(lits))
        z.extend(lits)
        z.extend((off & 255, off >> 8))
        if ml - 4 >= 15:
            _lz4_len(z, ml - 4)

    seq(chunk[0:x], x - y, 4)
    seq(chunk[x + 4:P3], P3 - P2, 8)                # planes 1 and 2 as literals, then a copy of plane 2
    seq(chunk[P3 + 8:P3 + 12], P3 + 12 - P1, 8)     # a copy of plane 1
    tail = chunk[P3 + 20:]
    z.append(min(len(tail), 15) << 4)
    if len(tail) >= 15:
        _lz4_len(z, len(tail))
    z.extend(tail)
    n, out = O.lz4_decompress(bytes(z), len(chunk))
    assert n == len(chunk) and out.tobytes() == bytes(chunk)
    data = torch.from_numpy(np.frombuffer(bytes(z) + bytes(64), np.uint8).copy()).cuda()
    off = torch.tensor([0, len(z)], dtype=torch.int64, device="cuda")
    dec = cz.decompress_field(data, off, (32, 32, 32), 1, True, encoder="lz4").cpu().numpy()
    ref = O.block_decompress(np.frombuffer(bytes(chunk[4:]), np.uint8), 1, 1)
    assert dec.tobytes() == ref.tobytes()
    assert cz.lz4_decompress(bytes(z), len(chunk)) == bytes(chunk)
