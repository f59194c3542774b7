"""The kernels' arithmetic and index maps, compiled for the host from the
same headers (tests/emu/cz_emu.cpp), against the oracle, bit for bit."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import blocks

HERE = os.path.dirname(os.path.abspath(__file__))
fp = C.POINTER(C.c_float)
u8p = C.POINTER(C.c_uint8)


@pytest.fixture(scope="module")
def emu():
    out_dir = os.path.join(HERE, "emu", "_build")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "libczemu.so")
    src = os.path.join(HERE, "emu", "cz_emu.cpp")
    hdr = [os.path.join(HERE, "..", "cubismz_gb300", "csrc", f) for f in ("cz_arith.cuh", "cz_line.cuh", "cz_layout.cuh")]
    if not os.path.exists(lib) or any(os.path.getmtime(p) > os.path.getmtime(lib) for p in hdr + [src]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", lib, src])
    L = C.CDLL(lib)
    L.emu_fwt.argtypes = [fp, C.c_int, C.c_void_p]
    L.emu_iwt.argtypes = [fp, C.c_int, C.c_void_p]
    L.emu_to_positional.argtypes = [fp, fp]
    L.emu_block_compress.argtypes = [fp, C.c_float, C.c_int, C.c_int, C.c_int, u8p, C.POINTER(C.c_int)]
    L.emu_block_decompress.argtypes = [u8p, C.c_int, C.c_int, C.c_int, fp]
    return L


def _edge_blocks():
    rng = np.random.default_rng(11)
    z = np.zeros((32, 32, 32), np.float32)
    out = [z, np.where(rng.random((32, 32, 32)) < 0.5, -0.0, 0.0).astype(np.float32)]
    sparse = z.copy()
    sparse[5, 6, 7] = 1e-3
    sparse[20, 1, 30] = -7.0
    out.append(sparse)
    out.append((rng.standard_normal(32 ** 3) * 10.0 ** rng.uniform(-8, 8, 32 ** 3)).astype(np.float32).reshape(32, 32, 32))
    tiny = (rng.standard_normal(32 ** 3) * 1e-39).astype(np.float32).reshape(32, 32, 32)  # subnormals
    out.append(tiny)
    huge = (rng.standard_normal(32 ** 3) * 1e36).astype(np.float32).reshape(32, 32, 32)
    out.append(huge)
    step = np.ones((32, 32, 32), np.float32)
    step[:, :, 16:] = 1e-30
    out.append(step)
    return out


def test_index_maps(emu):
    assert emu.emu_check_maps() == 0


@pytest.mark.parametrize("wtype", [1, 2, 3])
def test_emu_transform_bit_exact(emu, wtype, demo_field, small_field):
    bl = list(blocks(demo_field))[::5] + list(blocks(small_field))[::5] + _edge_blocks()
    for b in bl:
        phys = np.ascontiguousarray(b, np.float32).copy()
        emu.emu_fwt(phys.ctypes.data_as(fp), wtype, None)
        pos = np.zeros_like(phys)
        emu.emu_to_positional(phys.ctypes.data_as(fp), pos.ctypes.data_as(fp))
        want = O.fwt(b, wtype)
        assert np.array_equal(pos.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("wtype,zb,sh", [(1, 0, 0), (3, 4, 1), (2, 4, 0), (1, 0, 1)])
def test_emu_codec_bit_exact(emu, wtype, zb, sh, small_field):
    for b in list(blocks(small_field))[::11] + _edge_blocks()[:4]:
        for eps in (0.0, 1e-3, 0.05):
            out = np.zeros(4096 + 4 * 32768, np.uint8)
            n = C.c_int(0)
            emu.emu_block_compress(b.ctypes.data_as(fp), C.c_float(eps), wtype, zb, sh, out.ctypes.data_as(u8p),
                                   C.byref(n))
            rec = out[:n.value]
            assert np.array_equal(rec, O.block_compress(b, eps, wtype, zb, sh))
            dec = np.zeros((32, 32, 32), np.float32)
            assert emu.emu_block_decompress(rec.ctypes.data_as(u8p), rec.size, wtype, sh, dec.ctypes.data_as(fp)) == 0
            assert np.array_equal(dec.view(np.uint32), O.block_decompress(rec, wtype, sh).view(np.uint32))
