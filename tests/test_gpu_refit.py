"""The linear inverse transform, its hand-written adjoint and the
least-squares refit.

The adjoint is checked against the FP64 oracle (explicit transposes of the
1D inverse operators composed with the reference's sweeps), by the identity
<IWT c, y> = <c, IWT^T y> evaluated in FP64, and, through a
torch.autograd.Function whose backward is the adjoint, by central finite
differences (h = 1e-3) on a 64^3 subfield. The refit keeps the plain mask
and must give a higher PSNR at the same ratio."""
import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import blocks

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cz(gpu_lib):
    import cubismz_gb300 as cz
    return cz


def _stack(field):
    return np.stack(list(blocks(field)))


def _psnr(orig, dec):
    o = orig.astype(np.float64)
    mse = np.mean((dec.astype(np.float64) - o) ** 2)
    return 20 * np.log10((o.max() - o.min()) / (2 * np.sqrt(mse)))


@pytest.mark.parametrize("wtype", [1, 2, 3])
def test_iwt_linear_and_adjoint_match_fp64(cz, wtype):
    import torch
    rng = np.random.default_rng(10 + wtype)
    c = rng.standard_normal((4, 32, 32, 32)).astype(np.float32)
    y = rng.standard_normal((4, 32, 32, 32)).astype(np.float32)
    w = cz.iwt_linear(torch.from_numpy(c).cuda(), wtype).cpu().numpy()
    wt = cz.iwt_adjoint(torch.from_numpy(y).cuda(), wtype).cpu().numpy()
    for g in range(4):
        ref = O.iwt_f64(c[g], wtype)
        assert np.abs(w[g] - ref).max() <= 2e-5 * np.abs(ref).max()
        ref_t = O.iwt_adj_f64(y[g], wtype)
        assert np.abs(wt[g] - ref_t).max() <= 2e-5 * np.abs(ref_t).max()
    # <W c, y> = <c, W^T y>, both sides accumulated in FP64
    lhs = np.vdot(w.astype(np.float64), y.astype(np.float64))
    rhs = np.vdot(c.astype(np.float64), wt.astype(np.float64))
    assert abs(lhs - rhs) <= 1e-5 * np.sqrt(np.vdot(w, w) * np.vdot(y, y))


def test_iwt_linear_inverts_the_forward_transform(cz, small_field):
    """On real coefficients (the reference's fwt, positional layout) the
    binary32 linear inverse reproduces the block to binary32 accuracy."""
    import torch
    blk = _stack(small_field[:64, :64, :64])
    coef = np.stack([O.fwt(b, 1) for b in blk])
    back = cz.iwt_linear(torch.from_numpy(coef).cuda(), 1).cpu().numpy()
    assert np.abs(back - blk).max() <= 1e-5 * np.abs(blk).max()


def test_autograd_adjoint_finite_differences(cz, small_field):
    """torch.autograd.Function (test harness only) with the adjoint as its
    backward: gradients of 0.5 ||IWT(c) - x||^2 on a 64^3 subfield against
    central differences (h = 1e-3) of the GPU forward and of the FP64 oracle,
    and against the FP64 gradient IWT^T (IWT c - x)."""
    import torch

    class IWT(torch.autograd.Function):
        @staticmethod
        def forward(ctx, coef):
            return cz.iwt_linear(coef.contiguous(), 1)

        @staticmethod
        def backward(ctx, grad):
            return cz.iwt_adjoint(grad.contiguous(), 1)

    x = _stack(small_field[32:96, 32:96, 32:96])
    rng = np.random.default_rng(3)
    c0 = np.stack([O.fwt(b, 1) for b in x]) + 0.01 * rng.standard_normal(x.shape).astype(np.float32)
    xt = torch.from_numpy(x).cuda().double()
    c = torch.from_numpy(c0).cuda().requires_grad_(True)

    def loss_gpu(cc):
        return 0.5 * ((IWT.apply(cc).double() - xt) ** 2).sum()

    L = loss_gpu(c)
    L.backward()
    g = c.grad.cpu().numpy().astype(np.float64)
    # FP64 gradient from the oracle
    r64 = np.stack([O.iwt_f64(c0[k], 1) for k in range(len(x))]) - x.astype(np.float64)
    g64 = np.stack([O.iwt_adj_f64(r64[k], 1) for k in range(len(x))])
    assert np.abs(g - g64).max() <= 1e-4 * np.abs(g64).max()
    # directions: the gradient itself and two sparse random ones (64 entries)
    h = 1e-3
    gn = np.linalg.norm(g)
    dirs = [g / gn]
    for _ in range(2):
        v = np.zeros(x.shape)
        v.flat[rng.choice(v.size, 64, replace=False)] = rng.standard_normal(64)
        dirs.append(v / np.linalg.norm(v))

    def l64(cc):
        return 0.5 * sum(np.sum((O.iwt_f64(cc[j], 1) - x[j]) ** 2) for j in range(len(x)))

    for v in dirs:
        vt = torch.from_numpy(v.astype(np.float32)).cuda()
        with torch.no_grad():
            cp, cm = c + h * vt, c - h * vt
            fd = (loss_gpu(cp) - loss_gpu(cm)).item() / (2 * h)
            # the binary32 step actually taken; exact for a quadratic
            pred = float(np.vdot(g, (cp.double() - cm.double()).cpu().numpy())) / (2 * h)
        assert abs(fd - pred) <= 1e-3 * max(abs(pred), 1e-2 * gn), (fd, pred)
        fd64 = (l64(c0 + h * v) - l64(c0 - h * v)) / (2 * h)
        assert abs(fd64 - float(np.vdot(g, v))) <= 1e-4 * gn, (fd64, np.vdot(g, v))


def _records(cf):
    """Records of a stream compressed with encoder none, one block per chunk."""
    data, off = cf.to_device()
    d, o = data.cpu().numpy(), off.cpu().numpy()
    return [d[o[k] + 4:o[k + 1]] for k in range(len(o) - 1)]


@pytest.mark.parametrize("zb,shuffle,encoder", [(0, False, "none"), (4, True, "lz4")])
def test_refit_keeps_mask_and_raises_psnr(cz, small_field, zb, shuffle, encoder):
    import torch
    f = torch.from_numpy(small_field).cuda()
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    plain = cz.compress_field(f, eps, 1, zb, shuffle, encoder=encoder)
    pd, po = plain.to_device()
    refit = cz.refit_field(f, eps, iters=20, wtype=1, zerobits=zb, shuffle=shuffle, encoder=encoder)
    rd, ro = refit.to_device()
    assert refit.raw_bytes == plain.raw_bytes  # same mask, same survivor counts
    if encoder == "none":
        for a, b in zip(_records(plain), _records(refit)):
            assert len(a) == len(b) and np.array_equal(a[:4096], b[:4096])
    dec_p = cz.decompress_field(pd, po, small_field.shape, 1, shuffle, encoder=encoder).cpu().numpy()
    dec_r = cz.decompress_field(rd, ro, small_field.shape, 1, shuffle, encoder=encoder).cpu().numpy()
    # the refit stream is an ordinary stream: the restated reference decoder
    # reads it to the same bits
    enc = 1 if encoder == "lz4" else 0
    ref = O.field_decompress(rd.cpu().numpy(), ro.cpu().numpy(), small_field.shape, 1, int(shuffle), enc)
    assert np.array_equal(ref, dec_r)
    p_plain, p_refit = _psnr(small_field, dec_p), _psnr(small_field, dec_r)
    assert p_refit > p_plain + 0.1, (p_plain, p_refit)
    # identical record bytes before the lossless stage; LZ4 packs the refit
    # survivors' byte planes a little less tightly
    ratio_p, ratio_r = small_field.nbytes / plain.nbytes, small_field.nbytes / refit.nbytes
    assert abs(ratio_r / ratio_p - 1) < 0.05


def test_refit_with_zlib_encoder(cz, small_field):
    """Refit streams with Encoder: zlib: every chunk inflates with zlib to a
    record with the plain path's mask, the restated reference decoder reads
    the inflated records to the GPU's decode, and the refit PSNR is higher."""
    import zlib
    import torch
    f = torch.from_numpy(small_field).cuda()
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    refit = cz.refit_field(f, eps, iters=20, wtype=1, zerobits=4, shuffle=True, encoder="zlib")
    rd, ro = refit.to_device()
    hd, ho = rd.cpu().numpy().tobytes(), ro.cpu().numpy()
    recs = [zlib.decompress(hd[ho[c]:ho[c + 1]]) for c in range(len(ho) - 1)]
    for c, r in enumerate(recs):
        want = bytes(raw[roff[c]:roff[c + 1]])
        assert len(r) == len(want) and r[:4 + 4096] == want[:4 + 4096]  # header and mask
    rec_off = np.concatenate([[0], np.cumsum([len(r) for r in recs])]).astype(np.int64)
    ref = O.field_decompress(np.frombuffer(b"".join(recs), np.uint8), rec_off, small_field.shape, 1, 1)
    dec = cz.decompress_field(rd, ro, small_field.shape, 1, True, encoder="zlib").cpu().numpy()
    assert np.array_equal(ref, dec)
    plain = O.field_decompress(raw, roff, small_field.shape, 1, 1)
    assert _psnr(small_field, dec) > _psnr(small_field, plain) + 0.1
