"""The HDF5 tools' array layout (z fastest, interleaved channels, float or
double) to and from the codec's x-fastest field."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("nch,ch", [(1, 0), (3, 1)])
def test_zfastest_roundtrip(cz, dtype, nch, ch):
    import torch
    nx, ny, nz = 70, 40, 45
    g = torch.Generator(device="cuda").manual_seed(5)
    shape = (nx, ny, nz, nch) if nch > 1 else (nx, ny, nz)
    arr = torch.randn(shape, generator=g, device="cuda", dtype=getattr(torch, dtype))
    f = cz.field_from_zfastest(arr, channel=ch)
    src = arr[..., ch] if nch > 1 else arr
    want = src.permute(2, 1, 0).contiguous().float()  # (nz, ny, nx): x fastest
    assert torch.equal(f, want)
    out = torch.zeros(shape, device="cuda", dtype=torch.float32)
    cz.field_to_zfastest(f, out=out, channel=ch)
    back = out[..., ch] if nch > 1 else out
    assert torch.equal(back, src.float())
    if nch > 1:
        others = [k for k in range(nch) if k != ch]
        assert torch.count_nonzero(out[..., others]) == 0


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("shape", [(96, 40, 64), (32, 1, 32), (256, 7, 160)])
def test_zfastest_tiled_path(cz, dtype, shape):
    """Single-channel arrays with tile-multiple extents (the TMA tile path):
    both directions exact, every element placed once."""
    import torch
    nx, ny, nz = shape
    g = torch.Generator(device="cuda").manual_seed(11)
    arr = torch.randn(shape, generator=g, device="cuda", dtype=getattr(torch, dtype))
    f = cz.field_from_zfastest(arr)
    assert torch.equal(f, arr.permute(2, 1, 0).contiguous().float())
    out = torch.full(shape, float("nan"), device="cuda", dtype=torch.float32)
    cz.field_to_zfastest(f, out=out)
    assert torch.equal(out, arr.float())


def test_ingest_compress_egress(cz, small_field):
    """hdf2cz -> codec -> cz2hdf: the z-fastest array survives up to the
    codec's error, and equals the x-fastest path's decode."""
    import torch
    f = torch.from_numpy(small_field).cuda()
    zf = cz.field_to_zfastest(f)  # the tools' layout
    back = cz.field_from_zfastest(zf)
    assert torch.equal(back, f)
    cf = cz.compress_field(back, 1e-3, 1, 0, False, encoder="lz4")
    data, off = cf.to_device()
    dec = cz.decompress_field(data, off, small_field.shape, 1, False, encoder="lz4")
    out = cz.field_to_zfastest(dec)
    assert torch.equal(out, dec.permute(2, 1, 0).contiguous())
