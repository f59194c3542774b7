"""The GPU zlib encoder's serial part (cz_deflate.cuh), compiled for the
host: streams built from a parse decode with zlib to the input, under every
block coding; the predicted sizes are the written sizes; code lengths stay
within their limits and form complete codes."""
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
    lib = os.path.join(out_dir, "libczdeflate.so")
    src = os.path.join(HERE, "emu", "cz_deflate_emu.cpp")
    hdr = [os.path.join(HERE, "..", "cubismz_gb300", "csrc", f)
           for f in ("cz_deflate.cuh", "cz_inflate.cuh", "cz_arith.cuh")]
    if not os.path.exists(lib) or any(os.path.getmtime(p) > os.path.getmtime(lib) for p in hdr + [src]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", lib, src])
    L = C.CDLL(lib)
    L.emu_parse.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.emu_parse.restype = C.c_int
    L.emu_deflate.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                              C.c_longlong, C.c_void_p]
    L.emu_deflate.restype = C.c_longlong
    L.emu_huff_lengths.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.emu_huff_lengths.restype = C.c_int
    return L


def bound(n):
    return n + 6 * (n // 1024 + 2) + 8


def deflate(L, data, mode=-1, records=0, max_dist=32768, max_len=1 << 20):
    src = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
    seq = np.zeros(len(data) // 4 + 2, np.uint64)
    n = L.emu_parse(src.ctypes.data, len(data), max_dist, max_len, seq.ctypes.data, seq.size)
    assert n > 0
    cap = bound(len(data)) + len(data) // 2 + 64
    out = np.zeros(cap, np.uint8)
    nb = C.c_longlong(0)
    m = L.emu_deflate(src.ctypes.data, len(data), seq.ctypes.data, n, mode, records, out.ctypes.data, cap,
                      C.byref(nb))
    assert m > 0, m
    if mode == -1:
        assert m <= bound(len(data))
    return out[:m].tobytes(), nb.value


def samples(small_field):
    from oracle import czoracle as O
    rng = np.random.default_rng(3)
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    return [b"", b"a", b"ab", bytes(70000), bytes(259), bytes(260), bytes(261), bytes(516), bytes(517),
            rng.integers(0, 256, 50000, np.uint8).tobytes(), b"abcabcabd" * 3000,
            rng.integers(0, 5, 120000, np.uint8).tobytes(), rng.integers(0, 256, 200000, np.uint8).tobytes(),
            bytes(raw[off[0]:off[1]]), bytes(raw[off[0]:off[15]])]


@pytest.mark.parametrize("mode", [-1, 0, 1, 2])
def test_deflate_streams_decode_with_zlib(emu, mode, small_field):
    """Every block coding, blocks per 64 KiB; every block's written bits
    equal its counted bits (checked inside the emulation)."""
    for d in samples(small_field):
        z, _ = deflate(emu, d, mode)
        assert zlib.decompress(z) == d, (mode, len(d))


@pytest.mark.parametrize("bpc", [1, 15])
def test_record_chunks_split_per_plane(emu, small_field, bpc):
    """Chunks of shuffled block records: a block for the mask and each byte
    plane of every record; smaller than one block per chunk, and smaller
    than zlib's default level."""
    from oracle import czoracle as O
    raw, off = O.field_compress(small_field, 1e-3, 1, 4, 1, 0, 1)
    tot = ref = one = 0
    for c in range(0, 30, 3):
        d = bytes(raw[off[c]:off[min(c + bpc, len(off) - 1)]])
        z, nb = deflate(emu, d, -1, records=1)
        assert zlib.decompress(z) == d
        assert nb >= 4 * min(bpc, len(off) - 1 - c)
        tot += len(z)
        ref += len(zlib.compress(d, 6))
        one += len(deflate(emu, d, -1, records=0)[0])
    assert tot < one and tot < ref, (tot, one, ref)


def test_long_matches_are_split(emu):
    """Matches of any length (pieces of at most 258 bytes, none below 3)
    and distances at the 32 KiB limit."""
    rng = np.random.default_rng(5)
    unit = rng.integers(0, 256, 32768, np.uint8).tobytes()
    for n in (3, 258, 259, 260, 261, 515, 516, 517, 1000, 40000):
        d = unit + unit[:n] + rng.integers(0, 256, 100, np.uint8).tobytes()
        for mode in (1, 2):
            z, _ = deflate(emu, d, mode)
            assert zlib.decompress(z) == d, (n, mode)
    d = bytes(rng.integers(0, 3, 100000, np.uint8)) * 2
    for max_len in (4, 5, 258, 300):
        z, _ = deflate(emu, d, 2, max_len=max_len)
        assert zlib.decompress(z) == d


def test_huffman_lengths_limited_and_complete(emu):
    """Fibonacci weights force depths far past the limit; the limited code
    is complete (Kraft sum one) and keeps longer codes on smaller weights."""
    fib = [1, 1]
    while len(fib) < 40:
        fib.append(fib[-1] + fib[-2])
    rng = np.random.default_rng(9)
    cases = [np.array(fib[:n], np.uint32) for n in (2, 3, 16, 20, 30, 40)]
    cases += [np.sort(rng.integers(1, 1 << 20, n).astype(np.uint32)) for n in (2, 19, 30, 286)]
    cases += [np.ones(286, np.uint32), np.array([1] * 285 + [1 << 24], np.uint32)]
    for w in cases:
        for maxbits in (7, 15):
            if len(w) > (1 << maxbits):
                continue
            ln = np.zeros(len(w), np.uint8)
            assert emu.emu_huff_lengths(w.ctypes.data, len(w), maxbits, ln.ctypes.data) == 1
            assert ln.min() >= 1 and ln.max() <= maxbits
            assert sum(2.0 ** -int(x) for x in ln) == 1.0
            assert all(ln[i] >= ln[i + 1] for i in range(len(w) - 1))
