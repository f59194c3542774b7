"""The CPU oracle against the reference: its own sources built here
(oracle/_ref, skipped where the reference tree is absent) and the committed
golden fixtures (always)."""
import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import blocks, cz_size, header_text, res_line, seeded_blocks, sha, zlib_chunks


@pytest.mark.parametrize("case", range(12))
def test_oracle_matches_reference_block_hashes(golden, case):
    c = golden["block_cases"][case]
    for b, want_rec, want_dec in zip(seeded_blocks(), c["record_sha256"], c["decoded_sha256"]):
        rec = O.block_compress(b, c["eps"], c["wtype"], c["zerobits"], c["shuffle"])
        assert sha(rec) == want_rec
        assert sha(O.block_decompress(rec, c["wtype"], c["shuffle"]).tobytes()) == want_dec


def test_oracle_small_field_stream(golden, small_field):
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    assert int(off[-1]) == golden["small_field_raw_bytes"]
    assert sha(raw) == golden["small_field_raw_sha256"]


def test_oracle_reproduces_published_golden(golden, demo_field):
    """demo.h5, wtype 3, threshold 5e-5, zlib, 15-block chunks, 1 thread
    (Tests/Test1/test_wavz.sh:18,37,48) -> the published RES line."""
    raw, off = O.field_compress(demo_field, 5e-5, 3, 0, 0, 0, 1)
    z = zlib_chunks(raw, off, 15, 64)
    size = cz_size([len(c) for c in z], 64, header_text(4, 4, 4, 5e-5, "AverageInterpWavelet3rdOrder", "zlib"))
    assert size == golden["reference_rebuilt_cz_bytes"]
    dec = O.field_decompress(raw, off, demo_field.shape, 3)
    assert sha(dec.tobytes()) == golden["reference_demo_decoded_sha256"]
    assert res_line(demo_field, dec, size) == golden["published_res"]


def test_oracle_decodes_reference_lz4(golden):
    import os
    data = open(os.path.join(os.path.dirname(__file__), "golden", "ref_lz4_chunks.bin"), "rb").read()
    pos = 0
    for entry in golden["ref_lz4_chunks"]:
        zn, rn = np.frombuffer(data[pos:pos + 8], np.int32)
        z = data[pos + 8:pos + 8 + zn]
        pos += 8 + zn
        n, out = O.lz4_decompress(z, int(rn))
        assert n == rn == entry["raw_bytes"]
        assert sha(out) == entry["raw_sha256"]


def test_oracle_lz4_roundtrip_and_errors():
    rng = np.random.default_rng(5)
    for data in [b"", b"a", bytes(12), bytes(13), bytes(100000), rng.integers(0, 256, 70000, np.uint8).tobytes(),
                 (b"abcdefgh" * 3000) + rng.integers(0, 4, 5000, np.uint8).tobytes()]:
        z = O.lz4_compress(data)
        n, out = O.lz4_decompress(z, len(data))
        assert n == len(data) and out.tobytes() == data
    # truncated streams never decode to the full data (a prefix ending in a
    # literal run can itself be a valid, shorter stream)
    z = O.lz4_compress(bytes(5000) + b"xyz" * 100)
    for cut in (1, 2, 5, len(z) - 1):
        n, _ = O.lz4_decompress(z[:cut], 5300)
        assert n < 5300
    n, _ = O.lz4_decompress(z, 100)  # output too small
    assert n <= 0


def test_oracle_lz4_compress_reproduces_reference_chunks(golden):
    """The restated LZ4_compress gives the reference's own bytes for the
    committed chunks (records of the small field, LZ4_compressCtx: over 64
    KiB)."""
    import os
    from cubismz_gb300 import synth
    raw, off = O.field_compress(synth.config_field("small", 0), 1e-2, 1, 4, 1, 0, 1)
    data = open(os.path.join(os.path.dirname(__file__), "golden", "ref_lz4_chunks.bin"), "rb").read()
    pos = 0
    for entry in golden["ref_lz4_chunks"]:
        zn, rn = np.frombuffer(data[pos:pos + 8], np.int32)
        z = data[pos + 8:pos + 8 + zn]
        pos += 8 + zn
        chunk = raw[off[entry["chunk"]]:off[entry["chunk"] + 1]]
        assert sha(chunk) == entry["raw_sha256"] and len(chunk) == rn
        assert bytes(O.lz4_compress(chunk.tobytes())) == z


def test_oracle_lz4_decoder_matches_reference_cases():
    """The restated LZ4_uncompress_unknownOutputSize returns what the
    reference's own decoder returned (output size, or minus the input
    position of the error) on random, valid, edited and cut inputs, and the
    same output bytes."""
    from tests.helpers import lz4_cases
    seen = 0
    for data, cap, ref, ref_sha in lz4_cases():
        n, out = O.lz4_decompress(data, cap)
        assert n == ref, (len(data), cap, n, ref)
        if ref > 0:
            assert sha(out) == ref_sha
        seen += 1
    assert seen > 150


ref_missing = O.ref(0, 0, "none") is None


@pytest.mark.skipif(ref_missing, reason="reference sources not available on this machine")
@pytest.mark.parametrize("zb,sh", [(0, 0), (4, 1), (4, 0), (0, 1)])
def test_oracle_equals_reference_build(zb, sh, demo_field, small_field):
    L = O.ref(zb, sh, "none")
    rng = np.random.default_rng(zb * 10 + sh)
    bl = list(blocks(demo_field))[::7] + list(blocks(small_field))[::9]
    bl += [(rng.standard_normal(32 ** 3) * 10.0 ** rng.uniform(-20, 20)).astype(np.float32).reshape(32, 32, 32)]
    for wt in (1, 2, 3, 0):
        for b in bl:
            for eps in (0.0, 1e-4, 1e-2):
                r = O.ref_block_compress(L, b, eps, wt)
                assert np.array_equal(r, O.block_compress(b, eps, wt, zb, sh))
                d1 = O.ref_block_decompress(L, r, wt)
                assert np.array_equal(d1.view(np.uint32), O.block_decompress(r, wt, sh).view(np.uint32))


@pytest.mark.skipif(ref_missing, reason="reference sources not available on this machine")
def test_oracle_lz4_compress_equals_reference_build():
    """The restated LZ4_compress against the reference's, byte for byte:
    both table variants (under and over 65547 bytes), the end-of-input
    rules, runs, random and low-entropy bytes."""
    L = O.ref(4, 1, "lz4")
    rng = np.random.default_rng(12)
    cases = [b"", b"a", bytes(12), bytes(13), bytes(14), bytes(100000), rng.integers(0, 256, 70000, np.uint8).tobytes(),
             rng.integers(0, 3, 65546, np.uint8).tobytes(), rng.integers(0, 3, 65547, np.uint8).tobytes(),
             (b"abcdefgh" * 3000) + rng.integers(0, 4, 5000, np.uint8).tobytes()]
    cases += [rng.integers(0, 2, n, np.uint8).tobytes() for n in range(13, 40)]
    cases += [rng.integers(0, int(rng.integers(1, 256)), int(rng.integers(1, 3000)), np.uint8).tobytes()
              for _ in range(40)]
    for d in cases:
        assert bytes(O.lz4_compress(d)) == O.ref_lz4_compress(L, d).tobytes(), len(d)


@pytest.mark.skipif(ref_missing, reason="reference sources not available on this machine")
def test_oracle_lz4_streams_decode_with_reference_decoder(small_field):
    L = O.ref(4, 1, "lz4")
    raw, off = O.field_compress(small_field, 1e-2, 1, 4, 1, 0, 1)
    for c in range(0, len(off) - 1, 5):
        chunk = raw[off[c]:off[c + 1]]
        z = O.lz4_compress(chunk)
        n, out = O.ref_lz4_decompress(L, z, len(chunk))
        assert n == len(chunk) and np.array_equal(out, chunk)


@pytest.mark.skipif(ref_missing, reason="reference sources not available on this machine")
def test_fp64_oracle_is_close_to_binary32_path(small_field):
    b = next(blocks(small_field))
    for wt in (1, 3):
        c32 = O.fwt(b, wt)
        c64 = O.fwt_f64(b.astype(np.float64), wt)
        assert np.max(np.abs(c32 - c64)) < 1e-5
        back = O.iwt_f64(c64, wt)
        assert np.max(np.abs(back - b)) < 1e-12


@pytest.mark.parametrize("wtype", [1, 2, 3])
def test_fp64_adjoint_is_the_transpose(wtype):
    """The explicit-matrix adjoint of the FP64 inverse transform satisfies
    <IWT c, y> = <c, IWT^T y> and, column by column, (IWT^T y)_k = <IWT e_k, y>."""
    rng = np.random.default_rng(wtype)
    c = rng.standard_normal((32, 32, 32))
    y = rng.standard_normal((32, 32, 32))
    lhs = np.vdot(O.iwt_f64(c, wtype), y)
    rhs = np.vdot(c, O.iwt_adj_f64(y, wtype))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    adj = O.iwt_adj_f64(y, wtype).ravel()
    for k in [0, 5, 63, 64, 300, 511, 512, 4095, 4096, 20000, 32767]:
        e = np.zeros(32768)
        e[k] = 1.0
        assert abs(np.vdot(O.iwt_f64(e.reshape(32, 32, 32), wtype), y) - adj[k]) <= 1e-12 * (1 + abs(adj[k]))


@pytest.mark.parametrize("wtype", [1, 2, 3])
def test_fp64_inverse_matrices(wtype):
    """The explicit 1D inverse operators invert the reference's forward line
    transform (binary32 restatement, so to binary32 accuracy), and the FP64
    3D inverse inverts the FP64 forward."""
    for n in (8, 16, 32):
        M = O.inv_matrix(n, wtype)
        F = np.stack([O.transform1d(np.eye(n, dtype=np.float32)[j], wtype, True) for j in range(n)], axis=1)
        assert np.abs(M @ F.astype(np.float64) - np.eye(n)).max() < 1e-5
    x = np.random.default_rng(7).standard_normal((32, 32, 32))
    assert np.abs(O.iwt_f64(O.fwt_f64(x, wtype), wtype) - x).max() < 1e-12
