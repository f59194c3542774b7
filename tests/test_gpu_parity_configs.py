"""Bit-exact parity at the workloads' full sizes, every block compared.

* 512^3 field (200 blobs, 12 interfaces), wtype 1, zero-bits 4, shuffle,
  LZ4, thresholds 1e-4, 1e-3 and 1e-2 of the field's range: all 4096 block
  records and the whole pre-LZ4 stream equal the oracle's byte for byte,
  every LZ4 chunk decodes with the restated reference decoder to its
  record, and the GPU decode of the LZ4 stream equals the oracle's decode.
* 96 uneven fields (edges from {64, ..., 384}, thresholds log-uniform in
  [1e-5, 1e-2] of each field's range) through one captured plan launch:
  every field's chunks decode with the restated reference decoder to the
  oracle's records of that field, and the GPU decode equals the oracle's.
* The 256^3 refit field (threshold 1e-3): the refit keeps the plain path's
  mask in every record, and its records decode on the GPU exactly as the
  oracle decodes them.
* One 1024^3 field of the multi-field stress workload: every record and
  the decoded field.

The oracle (oracle/czoracle.c, OpenMP over blocks) restates the reference's
block loop (SerializerIO_WaveletCompression_MPI_Simple.h:187-345) and is
pinned to the reference build on CPU (tests/test_oracle.py)."""
import numpy as np
import pytest

from oracle import czoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


@pytest.fixture(scope="module")
def large():
    from cubismz_gb300 import synth
    return synth.config_field("large", 0)


def lz4_chunks_decode_to(data, off, raw, roff):
    """Every chunk c of (data, off) decodes with the restated reference
    decoder (LZ4_uncompress_unknownOutputSize) to raw[roff[c]:roff[c+1]]."""
    for c in range(len(off) - 1):
        want = raw[roff[c]:roff[c + 1]]
        n, out = O.lz4_decompress(data[off[c]:off[c + 1]], len(want))
        assert n == len(want) and np.array_equal(out, want), c


@pytest.mark.parametrize("rel", [1e-4, 1e-3, 1e-2])
def test_512_field_every_record(cz, large, rel):
    import torch
    eps = float(np.float32(rel * float(large.max() - large.min())))
    f = torch.from_numpy(large).cuda()
    raw, roff = O.field_compress(large, eps, 1, 4, 1, 0, 1)
    assert len(roff) == 4097
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="none")
    d, o = cf.to_device()
    assert np.array_equal(o.cpu().numpy(), roff)
    assert np.array_equal(d.cpu().numpy(), raw)  # all 4096 records, i.e. the pre-LZ4 stream
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="lz4")
    assert cf.raw_bytes == int(roff[-1])
    d, o = cf.to_device()
    lz4_chunks_decode_to(d.cpu().numpy(), o.cpu().numpy(), raw, roff)
    dec = cz.decompress_field(d, o, large.shape, 1, True, encoder="lz4").cpu().numpy()
    want = O.field_decompress(raw, roff, large.shape, 1, 1)
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))


def test_96_uneven_fields_one_plan(cz):
    import torch
    from cubismz_gb300 import synth
    shapes, thr = synth.batch_shapes(96, 0)
    fields = [synth.generate_torch(sh, seed=1000 + i, blobs=20, interfaces=3, device="cuda")
              for i, sh in enumerate(shapes)]
    eps = [float(np.float32(t * float(f.max() - f.min()))) for t, f in zip(thr, fields)]
    plan = cz.Plan(fields, eps, 1, 4, True, "lz4", tune=True)
    plan.launch()
    cf = plan.result()
    data, off = cf.to_device()
    data, off = data.cpu().numpy(), off.cpu().numpy()
    for i, (f, e) in enumerate(zip(fields, eps)):
        host = f.cpu().numpy()
        raw, roff = O.field_compress(host, e, 1, 4, 1, 0, 1)
        d, o = plan.field_chunks(data, off, i)
        lz4_chunks_decode_to(d, o, raw, roff)
        dec = cz.decompress_field(torch.from_numpy(np.ascontiguousarray(d)).cuda(), torch.from_numpy(o).cuda(),
                                  host.shape, 1, True, encoder="lz4").cpu().numpy()
        want = O.field_decompress(raw, roff, host.shape, 1, 1)
        assert np.array_equal(dec.view(np.uint32), want.view(np.uint32)), i
    plan.close()


def test_refit_field_mask_and_decode(cz):
    import torch
    from cubismz_gb300 import synth
    field = synth.config_field("refit", 0)
    f = torch.from_numpy(field).cuda()
    eps = 1e-3
    plain, poff = O.field_compress(field, eps, 1, 4, 1, 0, 1)
    rf = cz.refit_field(f, eps, 30, 1, 4, True, encoder="none")
    rd, ro = rf.to_device()
    rd, ro = rd.cpu().numpy(), ro.cpu().numpy()
    assert np.array_equal(ro, poff)  # same survivor counts per block
    for g in range(len(poff) - 1):
        # [int32 nbytes][4096-byte mask]: the plain path's mask
        assert np.array_equal(rd[ro[g]:ro[g] + 4100], plain[poff[g]:poff[g] + 4100]), g
    want = O.field_decompress(rd, ro, field.shape, 1, 1)
    rl = cz.refit_field(f, eps, 30, 1, 4, True, encoder="lz4")
    d, o = rl.to_device()
    lz4_chunks_decode_to(d.cpu().numpy(), o.cpu().numpy(), rd, ro)
    dec = cz.decompress_field(d, o, field.shape, 1, True, encoder="lz4").cpu().numpy()
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))
    # the refit lowers the error against the field where it matters
    e_plain = O.field_decompress(plain, poff, field.shape, 1, 1).astype(np.float64) - field
    e_refit = want.astype(np.float64) - field
    assert (e_refit ** 2).sum() < (e_plain ** 2).sum()


def test_1024_field_every_record(cz):
    """The multi-field stress workload's field size: one 1024^3 field (the
    density field's generator, evaluated on the GPU), threshold 1e-3 of its
    range, zero-bits 4, shuffle, LZ4 -- all 32768 records and the decoded
    field bit-exact to the oracle, every LZ4 chunk decoded by the restated
    reference decoder."""
    from cubismz_gb300 import synth
    f = synth.generate_torch((1024, 1024, 1024), seed=5000, blobs=400, interfaces=20, device="cuda")
    host = f.cpu().numpy()
    eps = float(np.float32(1e-3 * float(host.max() - host.min())))
    raw, roff = O.field_compress(host, eps, 1, 4, 1, 0, 1)
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="none")
    d, o = cf.to_device()
    assert np.array_equal(o.cpu().numpy(), roff)
    assert np.array_equal(d.cpu().numpy(), raw)
    del d, o
    cf = cz.compress_field(f, eps, 1, 4, True, encoder="lz4")
    d, o = cf.to_device()
    lz4_chunks_decode_to(d.cpu().numpy(), o.cpu().numpy(), raw, roff)
    dec = cz.decompress_field(d, o, host.shape, 1, True, encoder="lz4").cpu().numpy()
    want = O.field_decompress(raw, roff, host.shape, 1, 1)
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))
