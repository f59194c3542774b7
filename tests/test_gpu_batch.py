"""Batched uneven fields through one captured CUDA graph (a plan): every
field's records decode to the oracle's field, the tuned launch shape is one
of the candidates, and a relaunch after the fields change in place sees the
new contents."""
import numpy as np
import pytest

from oracle import czoracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(64, 96, 128), (96, 64, 64), (128, 128, 96), (32, 32, 32), (96, 64, 160)]
THR = [1e-5, 1e-4, 1e-3, 3e-3, 1e-2]


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


def test_plan_graph_batch(cz):
    import torch
    from cubismz_gb300 import synth
    fields = [synth.generate(s, seed=i, blobs=6, interfaces=2) for i, s in enumerate(SHAPES)]
    eps = [float(np.float32(t * (f.max() - f.min()))) for t, f in zip(THR, fields)]
    dev = [torch.from_numpy(f).cuda() for f in fields]
    plan = cz.Plan(dev, eps, wtype=1, zerobits=4, shuffle=True, encoder="lz4", tune=True)
    info = plan.info()
    assert info["lz4_warps_per_cta"] in (2, 4, 8, 16) and all(t > 0 for t in info["tune_ms"].values())
    # the tuned shape: the fastest LZ4 width and wavelet-kernel variant timed
    assert info["shape"]["lz4_chunks_per_cta"] == info["lz4_warps_per_cta"]
    assert all(t > 0 for t in info["lz4_stage_ms"].values())
    assert all(t > 0 for t in info["wavelet_kernel_ms"].values())
    lz = info["lz4_stage_ms"]
    assert lz[info["lz4_warps_per_cta"]] == min(lz.values())
    wk = info["wavelet_kernel_ms"]
    assert wk[("split_prefetch", "joint_prefetch")[info["shape"]["wavelet_variant"]]] == min(wk.values())

    def check(fs):
        for _ in range(2):
            plan.launch()
        cf = plan.result()
        data, off = cf.to_device()
        raw_total = 0
        for i, f in enumerate(fs):
            d, o = plan.field_chunks(data, off, i)
            dec = cz.decompress_field(d, o, f.shape, 1, True, encoder="lz4").cpu().numpy()
            raw, roff = O.field_compress(f, eps[i], 1, 4, 1, 0, 1)
            raw_total += int(roff[-1])
            assert np.array_equal(dec, O.field_decompress(raw, roff, f.shape, 1, 1))
        assert cf.raw_bytes == raw_total

    check(fields)
    dev[2].mul_(2.0)
    fields[2] = fields[2] * np.float32(2.0)
    check(fields)
    plan.close()


def test_plan_with_zlib_encoder(cz):
    """A plan with Encoder: zlib: every field's chunks inflate with zlib to
    the oracle's records, and the fields decode bit-exactly on the GPU."""
    import zlib
    import torch
    from cubismz_gb300 import synth
    fields = [synth.generate(s, seed=10 + i, blobs=6, interfaces=2) for i, s in enumerate(SHAPES)]
    eps = [float(np.float32(t * (f.max() - f.min()))) for t, f in zip(THR, fields)]
    dev = [torch.from_numpy(f).cuda() for f in fields]
    plan = cz.Plan(dev, eps, wtype=1, zerobits=4, shuffle=True, encoder="zlib", tune=True)
    plan.launch()
    cf = plan.result()
    data, off = cf.to_device()
    for i, f in enumerate(fields):
        d, o = plan.field_chunks(data, off, i)
        hd, ho = d.cpu().numpy().tobytes(), o.cpu().numpy()
        raw, roff = O.field_compress(f, eps[i], 1, 4, 1, 0, 1)
        for c in range(len(ho) - 1):
            assert zlib.decompress(hd[ho[c]:ho[c + 1]]) == bytes(raw[roff[c]:roff[c + 1]])
        dec = cz.decompress_field(d, o, f.shape, 1, True, encoder="zlib").cpu().numpy()
        assert np.array_equal(dec, O.field_decompress(raw, roff, f.shape, 1, 1))
    plan.close()


@pytest.mark.parametrize("encoder", ["lz4", "zlib", "none"])
def test_batch_compress_equals_single_fields(cz, encoder):
    """cz_batch_compress (one persistent launch over every field's blocks)
    gives each field the chunks that compressing it alone gives, and they
    decode to the oracle's field."""
    import torch
    from cubismz_gb300 import synth
    shapes = [(64, 96, 32), (32, 32, 160), (96, 64, 64)]
    thr = [1e-3, 1e-4, 1e-2]
    fields = [synth.generate(s, seed=20 + i, blobs=6, interfaces=2) for i, s in enumerate(shapes)]
    eps = [float(np.float32(t * (f.max() - f.min()))) for t, f in zip(thr, fields)]
    dev = [torch.from_numpy(f).cuda() for f in fields]
    got = [cf.to_device() for cf in cz.batch_compress(dev, eps, 1, 4, True, encoder=encoder)]
    for f, d_f, e, (d, o) in zip(fields, dev, eps, got):
        sd, so = cz.compress_field(d_f, e, 1, 4, True, encoder=encoder).to_device()
        assert torch.equal(o, so) and torch.equal(d, sd)
        dec = cz.decompress_field(d, o, f.shape, 1, True, encoder=encoder).cpu().numpy()
        ref = O.field_decompress(*O.field_compress(f, e, 1, 4, 1), f.shape, 1, 1)
        assert np.array_equal(dec, ref)


def test_threads_compress_concurrently(cz):
    """Host threads compress at the same time, each through its own
    context, and get the bytes a single thread gets."""
    import threading
    import torch
    from cubismz_gb300 import synth
    shapes = [(64, 64, 96), (32, 96, 64), (96, 32, 32), (64, 32, 64)]
    fields = [torch.from_numpy(synth.generate(s, seed=40 + i, blobs=6, interfaces=2)).cuda()
              for i, s in enumerate(shapes)]
    eps = [float(np.float32(1e-3 * float(f.max() - f.min()))) for f in fields]
    want = [cz.compress_field(f, e, 1, 4, True, encoder="lz4").to_device() for f, e in zip(fields, eps)]
    want = [(d.cpu(), o.cpu()) for d, o in want]
    got, errors = [None] * len(fields), []

    def work(i):
        try:
            torch.cuda.set_device(0)
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(3):
                    d, o = cz.compress_field(fields[i], eps[i], 1, 4, True, encoder="lz4", stream=s).to_device(s)
                s.synchronize()
            got[i] = (d.cpu(), o.cpu())
        except Exception as e:  # reported below
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(len(fields))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors
    for (wd, wo), (gd, go) in zip(want, got):
        assert torch.equal(wd, gd) and torch.equal(wo, go)

