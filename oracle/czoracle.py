"""ctypes bindings for the CPU oracle (libczoracle.so) and, where it was
built, for the reference's own codec (oracle/_ref/libczref_<variant>.so).

TEST INFRASTRUCTURE ONLY: imported by tests/ and __graft_entry__.smoke()
to check the GPU results, and by bench.py's CPU-baseline leg. The product
never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = {}

BS3 = 32 * 32 * 32
MASKBYTES = 4096
MAXRECORD = MASKBYTES + 4 * BS3

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i64p = C.POINTER(C.c_longlong)


def _p(a, t):
    return a.ctypes.data_as(t)


def lib():
    """Load (building on first use) the plain-C oracle."""
    global _LIB
    if _LIB is None:
        from oracle import build
        path = build.build_oracle()
        L = C.CDLL(path)
        L.czo_transform1d.argtypes = [_fp, C.c_int, C.c_int, C.c_int]
        L.czo_fwt.argtypes = [_fp, C.c_int]
        L.czo_iwt.argtypes = [_fp, C.c_int]
        L.czo_threshold.argtypes = [_fp, C.c_float, _u8p, _fp]
        L.czo_block_compress.argtypes = [_fp, C.c_float, C.c_int, C.c_int, C.c_int, _u8p, C.POINTER(C.c_int)]
        L.czo_block_decompress.argtypes = [_u8p, C.c_int, C.c_int, C.c_int, _fp]
        L.czo_fwt_f64.argtypes = [_dp, C.c_int]
        L.czo_iwt_f64.argtypes = [_dp, C.c_int]
        L.czo_inv_matrix.argtypes = [C.c_int, C.c_int, _dp]
        L.czo_iwt_adj_f64.argtypes = [_dp, C.c_int]
        L.czo_lz4_decompress.argtypes = [_u8p, C.c_int, _u8p, C.c_int]
        L.czo_lz4_compress.argtypes = [_u8p, C.c_int, _u8p, C.c_int]
        L.czo_lz4_bound.argtypes = [C.c_int]
        L.czo_field_compress.argtypes = [_fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int, C.c_int, _u8p, C.c_longlong, _i64p]
        L.czo_field_compress.restype = C.c_longlong
        L.czo_field_decompress.argtypes = [_u8p, _i64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_int, C.c_int, _fp]
        _LIB = L
    return _LIB


# ---------------------------------------------------------------- block codec
def fwt(block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float32).copy()
    lib().czo_fwt(_p(b, _fp), wtype)
    return b


def iwt(block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float32).copy()
    lib().czo_iwt(_p(b, _fp), wtype)
    return b


def fwt_f64(block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float64).copy()
    lib().czo_fwt_f64(_p(b, _dp), wtype)
    return b


def iwt_f64(block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float64).copy()
    lib().czo_iwt_f64(_p(b, _dp), wtype)
    return b


def inv_matrix(n, wtype):
    """The 1D inverse line operator of the FP64 restatement as an n x n matrix."""
    M = np.zeros((n, n), np.float64)
    lib().czo_inv_matrix(n, wtype, _p(M, _dp))
    return M


def iwt_adj_f64(block, wtype):
    """Adjoint of iwt_f64 (positional coefficient layout), from explicit matrices."""
    b = np.ascontiguousarray(block, dtype=np.float64).copy()
    lib().czo_iwt_adj_f64(_p(b, _dp), wtype)
    return b


def transform1d(line, wtype, fwd):
    x = np.ascontiguousarray(line, dtype=np.float32).copy()
    lib().czo_transform1d(_p(x, _fp), x.size, wtype, 1 if fwd else 0)
    return x


def block_compress(block, eps, wtype, zerobits=0, shuffle=0):
    b = np.ascontiguousarray(block, dtype=np.float32)
    out = np.zeros(MAXRECORD, np.uint8)
    n = C.c_int(0)
    lib().czo_block_compress(_p(b, _fp), C.c_float(eps), wtype, zerobits, shuffle, _p(out, _u8p), C.byref(n))
    return out[: n.value].copy()


def block_decompress(record, wtype, shuffle=0):
    r = np.ascontiguousarray(record, dtype=np.uint8)
    out = np.zeros((32, 32, 32), np.float32)
    rc = lib().czo_block_decompress(_p(r, _u8p), r.size, wtype, shuffle, _p(out, _fp))
    if rc != 0:
        raise ValueError(f"oracle rejected the record ({rc})")
    return out


def lz4_compress(data):
    d = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if not isinstance(data, np.ndarray) else data,
                             dtype=np.uint8)
    cap = lib().czo_lz4_bound(d.size)
    out = np.zeros(cap, np.uint8)
    n = lib().czo_lz4_compress(_p(d, _u8p), d.size, _p(out, _u8p), cap)
    return out[:n].copy()


def lz4_decompress(data, cap):
    d = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if not isinstance(data, np.ndarray) else data,
                             dtype=np.uint8)
    out = np.zeros(max(cap, 1), np.uint8)
    n = lib().czo_lz4_decompress(_p(d, _u8p), d.size, _p(out, _u8p), cap)
    return n, out[: max(n, 0)].copy()


# ---------------------------------------------------------------- field level
def field_compress(field, eps, wtype, zerobits=0, shuffle=0, encoder=0, blocks_per_chunk=1, nthreads=0):
    f = np.ascontiguousarray(field, dtype=np.float32)
    nz, ny, nx = f.shape
    nblocks = (nx // 32) * (ny // 32) * (nz // 32)
    nchunks = (nblocks + blocks_per_chunk - 1) // blocks_per_chunk
    cap = nblocks * (MAXRECORD + 4) + nchunks * 64 + 1024
    out = np.empty(cap, np.uint8)
    off = np.zeros(nchunks + 1, np.int64)
    n = lib().czo_field_compress(_p(f, _fp), nx, ny, nz, C.c_float(eps), wtype, zerobits, shuffle, encoder,
                                 blocks_per_chunk, nthreads, _p(out, _u8p), cap, _p(off, _i64p))
    if n < 0:
        raise RuntimeError("oracle field compression failed")
    return out[:n].copy(), off


def field_decompress(data, offsets, shape, wtype, shuffle=0, encoder=0, blocks_per_chunk=1, nthreads=0):
    nz, ny, nx = shape
    d = np.ascontiguousarray(data, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    out = np.zeros(shape, np.float32)
    rc = lib().czo_field_decompress(_p(d, _u8p), _p(off, _i64p), off.size - 1, nx, ny, nz, wtype, shuffle,
                                    encoder, blocks_per_chunk, nthreads, _p(out, _fp))
    if rc != 0:
        raise RuntimeError("oracle field decompression failed")
    return out


def max_threads():
    return lib().czo_max_threads()


# ------------------------------------------------------ reference (oracle/_ref)
def ref(zerobits=0, shuffle=0, encoder="none"):
    """The reference's own codec for one compile-time variant, or None when
    oracle/_ref was not built (no reference tree on this machine)."""
    name = f"zb{zerobits}_sh{1 if shuffle else 0}_{encoder}"
    if name in _REF:
        return _REF[name]
    path = os.path.join(HERE, "_ref", f"libczref_{name}.so")
    if not os.path.exists(path):
        from oracle import build
        if build.reference_available():
            build.build_ref()
    if not os.path.exists(path):
        _REF[name] = None
        return None
    L = C.CDLL(path)
    L.ref_block_compress.argtypes = [_fp, C.c_float, C.c_int, _u8p, C.POINTER(C.c_int)]
    L.ref_block_decompress.argtypes = [_u8p, C.c_int, C.c_int, _fp]
    L.ref_fwt.argtypes = [_fp, C.c_int]
    L.ref_iwt.argtypes = [_fp, C.c_int]
    L.ref_deflate_inplace.argtypes = [_u8p, C.c_uint, C.c_uint]
    L.ref_write_cz.argtypes = [_fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_char_p, C.c_int, C.c_int]
    L.ref_write_cz.restype = C.c_double
    L.ref_read_cz.argtypes = [C.c_char_p, C.c_int, _fp, C.POINTER(C.c_int)]
    if encoder == "lz4":
        L.ref_lz4_compress.argtypes = [_u8p, _u8p, C.c_int]
        L.ref_lz4_decompress.argtypes = [_u8p, _u8p, C.c_int, C.c_int]
    _REF[name] = L
    return L


def ref_block_compress(L, block, eps, wtype):
    b = np.ascontiguousarray(block, dtype=np.float32)
    out = np.zeros(MAXRECORD, np.uint8)
    n = C.c_int(0)
    L.ref_block_compress(_p(b, _fp), C.c_float(eps), wtype, _p(out, _u8p), C.byref(n))
    return out[: n.value].copy()


def ref_block_decompress(L, record, wtype):
    r = np.zeros(MAXRECORD + 16, np.uint8)
    r[: len(record)] = record
    out = np.zeros((32, 32, 32), np.float32)
    L.ref_block_decompress(_p(r, _u8p), len(record), wtype, _p(out, _fp))
    return out


def ref_fwt(L, block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float32).copy()
    L.ref_fwt(_p(b, _fp), wtype)
    return b


def ref_iwt(L, block, wtype):
    b = np.ascontiguousarray(block, dtype=np.float32).copy()
    L.ref_iwt(_p(b, _fp), wtype)
    return b


def ref_lz4_decompress(L, data, cap):
    d = np.zeros(len(data) + 16, np.uint8)
    d[: len(data)] = np.frombuffer(bytes(data), np.uint8)
    out = np.zeros(cap + 16, np.uint8)
    n = L.ref_lz4_decompress(_p(d, _u8p), _p(out, _u8p), len(data), cap)
    return n, out[: max(n, 0)].copy()


def ref_lz4_compress(L, data):
    d = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8))
    out = np.zeros(len(data) + len(data) // 255 + 16 + 16, np.uint8)
    n = L.ref_lz4_compress(_p(d, _u8p), _p(out, _u8p), len(data))
    return out[:n].copy()


def ref_deflate(L, data):
    buf = np.zeros(max(len(data), 64) + 1024, np.uint8)
    buf[: len(data)] = np.frombuffer(bytes(data), np.uint8)
    n = L.ref_deflate_inplace(_p(buf, _u8p), len(data), buf.size)
    return buf[:n].copy()


def ref_write_cz(L, field, eps, wtype, path, nthreads=1, repeats=1):
    f = np.ascontiguousarray(field, dtype=np.float32)
    nz, ny, nx = f.shape
    return L.ref_write_cz(_p(f, _fp), nx, ny, nz, C.c_float(eps), wtype,
                          path.encode() if path else None, nthreads, repeats)


def ref_read_cz(L, path, wtype):
    dims = (C.c_int * 3)()
    L.ref_read_cz(path.encode(), wtype, None, dims)
    out = np.zeros((dims[2], dims[1], dims[0]), np.float32)
    L.ref_read_cz(path.encode(), wtype, _p(out, _fp), dims)
    return out
