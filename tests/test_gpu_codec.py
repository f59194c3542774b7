"""GPU parity of the block codec (libczgpu.so) against the reference: the
committed reference hashes, the oracle bit for bit, and the published
golden line."""
import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import blocks, cz_size, header_text, res_line, seeded_blocks, sha, zlib_chunks

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


@pytest.mark.parametrize("case", range(12))
def test_block_records_match_reference_hashes(cz, golden, case):
    """WaveletCompressor::compress/decompress drop-in vs the reference's
    own outputs (hashes made by tests/golden/make_golden.py)."""
    c = golden["block_cases"][case]
    wc = cz.WaveletCompressor(zerobits=c["zerobits"], shuffle=bool(c["shuffle"]))
    for b, want_rec, want_dec in zip(seeded_blocks(), c["record_sha256"], c["decoded_sha256"]):
        wc.uncompressed_data()[...] = b
        n = wc.compress(c["eps"], False, c["wtype"])
        assert sha(wc.compressed_data()[:n]) == want_rec
        out = wc.decompress(False, n, c["wtype"])
        assert sha(out.tobytes()) == want_dec


@pytest.mark.parametrize("wtype,zb,sh,eps", [(1, 0, 0, 1e-3), (3, 4, 1, 1e-3), (2, 0, 1, 0.0), (3, 0, 0, 5e-5)])
def test_field_stream_bit_exact(cz, torch_cuda, small_field, wtype, zb, sh, eps):
    """Whole-field records (one per chunk, no lossless stage) equal the
    oracle's byte for byte; the decoded field equals the oracle's."""
    torch = torch_cuda
    f = torch.from_numpy(small_field).cuda()
    cf = cz.compress_field(f, eps, wtype, zb, sh, encoder="none")
    data, off = cf.to_device()
    raw, ooff = O.field_compress(small_field, eps, wtype, zb, sh, 0, 1)
    assert np.array_equal(off.cpu().numpy(), ooff)
    assert np.array_equal(data.cpu().numpy(), raw)
    dec = cz.decompress_field(data, off, small_field.shape, wtype, sh, encoder="none")
    want = O.field_decompress(raw, ooff, small_field.shape, wtype, sh)
    assert np.array_equal(dec.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_published_golden_from_gpu_records(cz, torch_cuda, golden, demo_field):
    """demo.h5, wtype 3, threshold 5e-5: the GPU records, grouped in the
    reference's 15-block chunks and deflated as the zlib build does, give
    the published RES line; the GPU decoder gives the reference's field."""
    torch = torch_cuda
    f = torch.from_numpy(demo_field).cuda()
    cf = cz.compress_field(f, 5e-5, 3, 0, False, encoder="none")
    data, off = cf.to_device()
    raw, roff = data.cpu().numpy(), off.cpu().numpy()
    z = zlib_chunks(raw, roff, 15, 64)
    size = cz_size([len(c) for c in z], 64, header_text(4, 4, 4, 5e-5, "AverageInterpWavelet3rdOrder", "zlib"))
    assert size == golden["reference_rebuilt_cz_bytes"]
    dec = cz.decompress_field(data, off, demo_field.shape, 3, False, encoder="none").cpu().numpy()
    assert sha(dec.tobytes()) == golden["reference_demo_decoded_sha256"]
    assert res_line(demo_field, dec, size) == golden["published_res"]


def test_blocks_per_chunk_grouping(cz, torch_cuda, small_field):
    torch = torch_cuda
    f = torch.from_numpy(small_field).cuda()
    for bpc in (3, 15):
        cf = cz.compress_field(f, 1e-3, 1, 4, True, encoder="none", blocks_per_chunk=bpc)
        data, off = cf.to_device()
        raw, ooff = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, bpc)
        assert np.array_equal(off.cpu().numpy(), ooff)
        assert np.array_equal(data.cpu().numpy(), raw)
        dec = cz.decompress_field(data, off, small_field.shape, 1, True, encoder="none", blocks_per_chunk=bpc)
        assert np.array_equal(dec.cpu().numpy(), O.field_decompress(raw, ooff, small_field.shape, 1, 1, 0, bpc))


def test_edge_blocks(cz):
    rng = np.random.default_rng(3)
    z = np.zeros((32, 32, 32), np.float32)
    cases = [z, np.where(rng.random((32, 32, 32)) < 0.5, -0.0, 0.0).astype(np.float32),
             (rng.standard_normal(32 ** 3) * 10.0 ** rng.uniform(-8, 8, 32 ** 3)).astype(np.float32).reshape(32, 32, 32),
             (rng.standard_normal(32 ** 3) * 1e-39).astype(np.float32).reshape(32, 32, 32),
             (rng.standard_normal(32 ** 3) * 1e36).astype(np.float32).reshape(32, 32, 32)]
    for wt in (1, 2, 3):
        wc = cz.WaveletCompressor(zerobits=0, shuffle=False)
        for b in cases:
            for eps in (0.0, 1e-3, -1.0):
                wc.uncompressed_data()[...] = b
                n = wc.compress(eps, False, wt)
                want = O.block_compress(b, eps, wt, 0, 0)
                assert np.array_equal(wc.compressed_data()[:n], want)
                out = wc.decompress(False, n, wt)
                assert np.array_equal(out.view(np.uint32), O.block_decompress(want, wt, 0).view(np.uint32))


def test_corrupt_records_are_rejected(cz):
    wc = cz.WaveletCompressor()
    b = np.random.default_rng(0).standard_normal((32, 32, 32)).astype(np.float32)
    wc.uncompressed_data()[...] = b
    n = wc.compress(0.5, False, 1)
    wc.compressed_data()[0] = 0  # clear coarse mask bits: count and base case no longer agree
    with pytest.raises(cz.CzError):
        wc.decompress(False, n, 1)
    wc.compressed_data()[0] = 0xFF
    with pytest.raises(cz.CzError):
        wc.decompress(False, n - 8, 1)


def test_misaligned_field_is_refused(cz, torch_cuda):
    """A contiguous field view that does not start on a 16-byte boundary is
    refused with CZ_E_ARG before any launch (rows are read as 16-byte
    vectors), and the context keeps working."""
    torch = torch_cuda
    from cubismz_gb300._lib import CzError, CZ_E_ARG
    buf = torch.zeros(32 ** 3 + 4, dtype=torch.float32, device="cuda")
    view = buf[1:1 + 32 ** 3].view(32, 32, 32)
    assert view.is_contiguous() and view.data_ptr() % 16 == 4
    with pytest.raises(CzError) as e:
        cz.compress_field(view, 1e-3, 1, 0, False, encoder="lz4")
    assert e.value.code == CZ_E_ARG
    good = buf[4:4 + 32 ** 3].view(32, 32, 32)
    cf = cz.compress_field(good, 1e-3, 1, 0, False, encoder="lz4")
    data, off = cf.to_device()
    with pytest.raises(CzError) as e:
        cz.decompress_field(data, off, (32, 32, 32), 1, False, encoder="lz4", out=view)
    assert e.value.code == CZ_E_ARG
    dec = cz.decompress_field(data, off, (32, 32, 32), 1, False, encoder="lz4").cpu().numpy()
    assert np.array_equal(dec, np.zeros((32, 32, 32), np.float32))
