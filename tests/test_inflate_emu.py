"""The GPU zlib decoder's serial part (cz_inflate.cuh), compiled for the
host, against zlib: every block type and level decodes to zlib's output,
malformed streams are rejected where zlib rejects them."""
import ctypes as C
import os
import subprocess
import zlib

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def emu():
    out_dir = os.path.join(HERE, "emu", "_build")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "libczinflate.so")
    src = os.path.join(HERE, "emu", "cz_inflate_emu.cpp")
    hdr = [os.path.join(HERE, "..", "cubismz_gb300", "csrc", f) for f in ("cz_inflate.cuh", "cz_arith.cuh")]
    if not os.path.exists(lib) or any(os.path.getmtime(p) > os.path.getmtime(lib) for p in hdr + [src]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", lib, src])
    L = C.CDLL(lib)
    L.emu_inflate.argtypes = [C.c_char_p, C.c_longlong, C.c_void_p, C.c_longlong]
    L.emu_inflate.restype = C.c_longlong
    return L


def inflate(L, z, cap):
    out = np.zeros(max(cap, 1), np.uint8)
    n = L.emu_inflate(z, len(z), out.ctypes.data, cap)
    return None if n < 0 else out[:n].tobytes()



@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_inflate_matches_zlib(emu, level, small_field):
    from oracle import czoracle as O
    rng = np.random.default_rng(level)
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    samples = [b"", b"a", bytes(70000), rng.integers(0, 256, 50000, np.uint8).tobytes(),
               b"abcabcabd" * 3000, rng.integers(0, 5, 120000, np.uint8).tobytes(), bytes(raw[off[0]:off[15]])]
    for d in samples:
        for strategy in (zlib.Z_DEFAULT_STRATEGY, zlib.Z_FIXED, zlib.Z_FILTERED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE):
            co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
            z = co.compress(d) + co.flush()
            assert inflate(emu, z, len(d)) == d, (level, strategy, len(d))


def test_inflate_rejects_like_zlib(emu):
    rng = np.random.default_rng(7)
    d = rng.integers(0, 8, 30000, np.uint8).tobytes()
    z = zlib.compress(d, 6)
    for b in (z[:len(z) // 2], z[:-1], z[:-4] + bytes(4), b"\x00\x00", z[2:]):
        assert inflate(emu, b, len(d)) is None
    assert inflate(emu, z, len(d) - 1) is None
    agree = 0
    for _ in range(400):
        junk = bytes([0x78, 0x9c]) + rng.integers(0, 256, int(rng.integers(1, 400)), np.uint8).tobytes()
        try:
            want = zlib.decompress(junk)
        except zlib.error:
            want = None
        if want is not None and len(want) > 65536:
            want = None
        assert inflate(emu, junk, 65536) == want
        agree += 1
    assert agree == 400


def edited_streams(seed=11, per=25):
    """Valid streams (dynamic, fixed and stored blocks) with one byte
    changed, seeded."""
    rng = np.random.default_rng(seed)
    d = (rng.integers(0, 6, 20000, np.uint8).tobytes() + bytes(3000) + b"pattern-" * 400
         + rng.integers(0, 256, 2000, np.uint8).tobytes())
    streams = [zlib.compress(d, 6), zlib.compress(d, 1), zlib.compress(d, 0)]
    co = zlib.compressobj(9, zlib.DEFLATED, 15, 9, zlib.Z_FIXED)
    streams.append(co.compress(d) + co.flush())
    for z in streams:
        for _ in range(per):
            e = bytearray(z)
            pos = int(rng.integers(0, len(z)))
            e[pos] = (e[pos] + int(rng.integers(1, 256))) & 255
            yield bytes(e), len(d)


def test_inflate_edited_streams_like_zlib(emu):
    for e, cap in edited_streams(per=60):
        try:
            want = zlib.decompress(e)
        except zlib.error:
            want = None
        if want is not None and len(want) > cap:
            want = None
        assert inflate(emu, e, cap) == want

