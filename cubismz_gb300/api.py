"""Python mirror of the reference compressor interface over libczgpu.so.

The names follow the reference: WaveletCompressor mirrors
WaveletCompressorGeneric<32,float> (Compressor/source/WaveletCompressor.h:35-94):
uncompressed_data(), compress(threshold, float16, wtype), compressed_data(),
decompress(float16, nbytes, wtype). Field-level calls take torch CUDA
tensors (device memory) or numpy arrays (host memory); torch is plumbing for
device memory and streams only. Errors raise CzError, as the reference
aborts.
"""
import ctypes as C
import threading

import numpy as np

from . import _lib
from ._lib import CzError, Params, Stream

_TLS = threading.local()  # contexts per host thread: a context's calls must not overlap


class Context:
    """One libczgpu context (device scratch buffers grow on demand)."""

    def __init__(self, device=0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.cz_create(device, C.byref(h))
        if rc != 0:
            raise CzError(rc, f"cz_create({device}) failed (no CUDA device?)")
        self.h = h
        self.device = device

    def check(self, rc):
        if rc != 0:
            raise CzError(rc, self.L.cz_last_error(self.h).decode(errors="replace"))

    def set_timing(self, on=True):
        self.check(self.L.cz_set_timing(self.h, 1 if on else 0))

    def set_lz4_effort(self, effort):
        """Parse effort of the LZ4 encoder for later calls: 0 fastest, 1
        (default) with backward match extension, 2 most matches."""
        self.check(self.L.cz_set_lz4_effort(self.h, int(effort)))

    def stage_times(self):
        """Per-stage device times (ms) of the last field call."""
        out = (C.c_float * 3)()
        n = self.L.cz_stage_times(self.h, out, 3)
        return list(out)[:max(n, 0)]

    def close(self):
        if self.h:
            self.L.cz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def context(device=0):
    """This host thread's context on `device` (each thread has its own, as
    each OpenMP thread of the reference has its own compressor)."""
    ctxs = getattr(_TLS, "ctxs", None)
    if ctxs is None:
        ctxs = _TLS.ctxs = {}
    if device not in ctxs:
        ctxs[device] = Context(device)
    return ctxs[device]


def params(eps, wtype=1, zerobits=0, shuffle=False, encoder="none", blocks_per_chunk=1):
    enc = {"none": _lib.ENCODER_NONE, "lz4": _lib.ENCODER_LZ4, "zlib": _lib.ENCODER_ZLIB}[encoder] \
        if isinstance(encoder, str) else int(encoder)
    return Params(float(eps), int(wtype), int(zerobits), 1 if shuffle else 0, enc, int(blocks_per_chunk))


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _f32(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class WaveletCompressor:
    """Per-block drop-in for WaveletCompressorGeneric<32,float>: the same
    method names and buffer semantics; compression runs on the GPU.
    zerobits/shuffle are the reference's build options (-D_ZEROBITS_,
    -D_USE_SHUFFLE3_) given at construction."""

    def __init__(self, zerobits=0, shuffle=False, device=0):
        self.ctx = context(device)
        self.zerobits = zerobits
        self.shuffle = shuffle
        self._data = np.zeros((32, 32, 32), np.float32)
        self._buf = np.zeros(_lib.MAX_RECORD, np.uint8)

    def uncompressed_data(self):
        return self._data

    def compressed_data(self):
        return self._buf

    def compress(self, threshold, float16=False, wtype=1):
        n = C.c_int(0)
        d = np.ascontiguousarray(self._data, np.float32)
        self.ctx.check(self.ctx.L.cz_block_compress(self.ctx.h, _f32(d), C.c_float(threshold), int(wtype),
                                                    self.zerobits, 1 if self.shuffle else 0, _u8(self._buf),
                                                    C.byref(n)))
        return n.value

    def decompress(self, float16, nbytes, wtype, out=None):
        dst = np.zeros((32, 32, 32), np.float32) if out is None else out
        self.ctx.check(self.ctx.L.cz_block_decompress(self.ctx.h, _u8(self._buf), int(nbytes), int(wtype),
                                                      1 if self.shuffle else 0, _f32(dst)))
        self._data[...] = dst
        return dst


def lz4_compress(data, device=0):
    """LZ4_compress on the GPU (host bytes in, host bytes out)."""
    ctx = context(device)
    src = np.frombuffer(bytes(data), np.uint8).copy()
    cap = ctx.L.cz_lz4_bound(src.size)
    dst = np.zeros(max(cap, 1), np.uint8)
    n = C.c_int(0)
    ctx.check(ctx.L.cz_lz4_compress(ctx.h, _u8(src) if src.size else None, src.size, _u8(dst), cap, C.byref(n)))
    return dst[: n.value].tobytes()


def lz4_decompress(data, cap, device=0):
    """LZ4_uncompress_unknownOutputSize semantics; raises CzError on
    malformed input."""
    ctx = context(device)
    src = np.frombuffer(bytes(data), np.uint8).copy()
    dst = np.zeros(max(cap, 1), np.uint8)
    n = C.c_int(0)
    rc = ctx.L.cz_lz4_decompress(ctx.h, _u8(src) if src.size else None, src.size, _u8(dst), cap, C.byref(n))
    ctx.check(rc)
    return dst[: n.value].tobytes()


def zlib_compress(data, device=0):
    """deflate_inplace's zlib branch on the GPU (host bytes in, a zlib
    stream out; any inflate reads it)."""
    ctx = context(device)
    src = np.frombuffer(bytes(data), np.uint8).copy()
    cap = ctx.L.cz_zlib_bound(src.size)
    dst = np.zeros(max(cap, 1), np.uint8)
    n = C.c_int(0)
    ctx.check(ctx.L.cz_zlib_compress(ctx.h, _u8(src) if src.size else None, src.size, _u8(dst), cap, C.byref(n)))
    return dst[: n.value].tobytes()


def zlib_decompress(data, cap, device=0):
    """zdecompress's zlib branch on the GPU; raises CzError on malformed
    input (the Adler-32 trailer is checked)."""
    ctx = context(device)
    src = np.frombuffer(bytes(data), np.uint8).copy()
    dst = np.zeros(max(cap, 1), np.uint8)
    n = C.c_int(0)
    rc = ctx.L.cz_zlib_decompress(ctx.h, _u8(src) if src.size else None, src.size, _u8(dst), cap, C.byref(n))
    ctx.check(rc)
    return dst[: n.value].tobytes()


class CompressedField:
    """A compressed field in the context's device buffers (valid until the
    next call on the same context)."""

    def __init__(self, ctx, stream, shape, prm):
        self.ctx, self.s, self.shape, self.params = ctx, stream, shape, prm

    @property
    def nbytes(self):
        return self.s.data_bytes

    @property
    def raw_bytes(self):
        return self.s.raw_bytes

    def to_device(self, stream=None):
        """Copy the compressed chunks and their offsets (rebased to 0) into
        new CUDA tensors (uint8 data, int64 offsets)."""
        import torch
        dev = f"cuda:{self.ctx.device}"
        data = torch.empty(max(self.s.data_bytes, 1), dtype=torch.uint8, device=dev)
        off = torch.empty(self.s.nchunks + 1, dtype=torch.int64, device=dev)
        st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        self.ctx.check(self.ctx.L.cz_stream_copy(self.ctx.h, C.byref(self.s), C.c_void_p(data.data_ptr()),
                                                 C.c_void_p(off.data_ptr()), C.c_void_p(st)))
        return data[: self.s.data_bytes], off

    def image(self):
        """The .cz file image (host bytes)."""
        nz, ny, nx = self.shape
        cap = self.ctx.L.cz_file_bytes(self.ctx.h, C.byref(self.s), nx, ny, nz, C.byref(self.params))
        out = np.empty(cap, np.uint8)
        w = C.c_longlong(0)
        self.ctx.check(self.ctx.L.cz_file_image(self.ctx.h, C.byref(self.s), nx, ny, nz, C.byref(self.params),
                                                out.ctypes.data, cap, C.byref(w)))
        return out[: w.value].tobytes()


def compress_field(field, eps, wtype=1, zerobits=0, shuffle=False, encoder="lz4", blocks_per_chunk=1, stream=None):
    """Compress a CUDA tensor field of shape (nz, ny, nx), x fastest."""
    import torch
    assert field.is_cuda and field.dtype == torch.float32 and field.is_contiguous()
    nz, ny, nx = field.shape
    ctx = context(field.device.index or 0)
    prm = params(eps, wtype, zerobits, shuffle, encoder, blocks_per_chunk)
    s = Stream()
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(field.device).cuda_stream
    ctx.check(ctx.L.cz_field_compress(ctx.h, C.c_void_p(field.data_ptr()), nx, ny, nz, C.byref(prm),
                                      C.c_void_p(st), C.byref(s)))
    return CompressedField(ctx, s, (nz, ny, nx), prm)


def batch_compress(fields, eps, wtype=1, zerobits=0, shuffle=False, encoder="lz4", stream=None):
    """cz_batch_compress: CUDA fields of uneven (nz, ny, nx) extents, one
    threshold each, in one persistent wavelet launch over all their blocks
    (one record per chunk). Returns a CompressedField per field; they share
    the context's device buffers (valid until the next call on it)."""
    import torch
    for f in fields:
        assert f.is_cuda and f.dtype == torch.float32 and f.is_contiguous()
    n = len(fields)
    dev = fields[0].device
    ctx = context(dev.index or 0)
    ptrs = (C.c_void_p * n)(*[f.data_ptr() for f in fields])
    dims = (C.c_int * (3 * n))(*[d for f in fields for d in (f.shape[2], f.shape[1], f.shape[0])])
    e = (C.c_float * n)(*[float(x) for x in eps])
    prm = params(0.0, wtype, zerobits, shuffle, encoder, 1)
    outs = (Stream * n)()
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    ctx.check(ctx.L.cz_batch_compress(ctx.h, n, ptrs, dims, e, C.byref(prm), C.c_void_p(st), outs))
    res = []
    for i, f in enumerate(fields):
        s = Stream(outs[i].data, outs[i].data_bytes, outs[i].chunk_offsets, outs[i].nchunks, outs[i].nblocks,
                   outs[i].raw_bytes)
        # a field's size is its last rebased chunk offset
        off = torch.empty(s.nchunks + 1, dtype=torch.int64, device=dev)
        ctx.check(ctx.L.cz_stream_copy(ctx.h, C.byref(s), None, C.c_void_p(off.data_ptr()), C.c_void_p(st)))
        s.data_bytes = int(off[-1].item())
        res.append(CompressedField(ctx, s, tuple(f.shape), prm))
    return res


class Plan:
    """A batch of CUDA fields (shape (nz, ny, nx), float32, contiguous) with
    per-field thresholds, compressed by one captured CUDA graph (one
    persistent wavelet launch over all fields' blocks, then the LZ4 stage
    and the stream assembly); the LZ4 launch shape is tuned on the batch
    when `tune` is set. Field contents may change between launches."""

    def __init__(self, fields, eps, wtype=1, zerobits=0, shuffle=False, encoder="lz4", tune=True):
        import torch
        for f in fields:
            assert f.is_cuda and f.dtype == torch.float32 and f.is_contiguous()
        self.fields = list(fields)
        self.ctx = context(self.fields[0].device.index or 0)
        n = len(self.fields)
        ptrs = (C.c_void_p * n)(*[f.data_ptr() for f in self.fields])
        dims = (C.c_int * (3 * n))(*[d for f in self.fields for d in (f.shape[2], f.shape[1], f.shape[0])])
        e = (C.c_float * n)(*[float(x) for x in eps])
        self.prm = params(0.0, wtype, zerobits, shuffle, encoder, 1)
        self.h = C.c_void_p()
        self.ctx.check(self.ctx.L.cz_plan_create(self.ctx.h, n, ptrs, dims, e, C.byref(self.prm), int(bool(tune)),
                                                 C.byref(self.h)))
        self.nblocks = [(f.shape[0] // 32) * (f.shape[1] // 32) * (f.shape[2] // 32) for f in self.fields]

    def launch(self, stream=None):
        import torch
        st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(self.fields[0].device).cuda_stream
        rc = self.ctx.L.cz_plan_launch(self.h, C.c_void_p(st))
        if rc != 0:
            raise CzError(rc, "graph launch failed")

    def result(self, stream=None):
        """The batch's stream (CompressedField over all fields' chunks)."""
        import torch
        st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(self.fields[0].device).cuda_stream
        s = Stream()
        rc = self.ctx.L.cz_plan_result(self.h, C.c_void_p(st), C.byref(s), None)
        if rc != 0:
            raise CzError(rc, self.ctx.L.cz_plan_last_error(self.h).decode())
        return CompressedField(self.ctx, s, None, self.prm)

    def field_chunks(self, data, offsets, i):
        """Field i's chunks out of the batch's (data, offsets) from to_device()."""
        b0 = sum(self.nblocks[:i])
        o = offsets[b0:b0 + self.nblocks[i] + 1]
        return data[int(o[0]):int(o[-1])], o - o[0]

    def info(self):
        w = C.c_int(0)
        t = (C.c_float * 3)()
        self.ctx.L.cz_plan_info(self.h, C.byref(w), t)
        shape = (C.c_int * 2)()
        ms = (C.c_float * 6)()
        self.ctx.L.cz_plan_shape(self.h, shape, ms)
        return {"lz4_warps_per_cta": w.value, "tune_ms": {2: t[0], 4: t[1], 8: t[2]},
                "shape": {"lz4_chunks_per_cta": shape[0], "wavelet_variant": shape[1]},
                "lz4_stage_ms": {2: ms[0], 4: ms[1], 8: ms[2], 16: ms[3]},
                "wavelet_kernel_ms": {"split_prefetch": ms[4], "joint_prefetch": ms[5]}}

    def close(self):
        if self.h:
            self.ctx.L.cz_plan_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def refit_field(field, eps, iters=30, wtype=1, zerobits=0, shuffle=False, encoder="lz4", blocks_per_chunk=1,
                stream=None):
    """compress_field with the retained coefficients refit by `iters` CGLS
    steps per block (same mask, same stream layout)."""
    import torch
    assert field.is_cuda and field.dtype == torch.float32 and field.is_contiguous()
    nz, ny, nx = field.shape
    ctx = context(field.device.index or 0)
    prm = params(eps, wtype, zerobits, shuffle, encoder, blocks_per_chunk)
    s = Stream()
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(field.device).cuda_stream
    ctx.check(ctx.L.cz_refit(ctx.h, C.c_void_p(field.data_ptr()), nx, ny, nz, C.byref(prm), int(iters),
                             C.c_void_p(st), C.byref(s)))
    return CompressedField(ctx, s, (nz, ny, nx), prm)


def _blocks_op(name, src, wtype, stream):
    import torch
    assert src.is_cuda and src.dtype == torch.float32 and src.is_contiguous() and src.numel() % 32768 == 0
    ctx = context(src.device.index or 0)
    out = torch.empty_like(src)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(src.device).cuda_stream
    ctx.check(getattr(ctx.L, name)(ctx.h, C.c_void_p(src.data_ptr()), src.numel() // 32768, int(wtype),
                                   C.c_void_p(out.data_ptr()), C.c_void_p(st)))
    return out


def iwt_linear(coef, wtype=1, stream=None):
    """Inverse transform (binary32 linear map) of stacked 32^3 coefficient
    blocks in the reference's positional layout -> stacked sample blocks."""
    return _blocks_op("cz_iwt_linear", coef, wtype, stream)


def iwt_adjoint(blocks, wtype=1, stream=None):
    """Adjoint of iwt_linear: stacked sample blocks -> positional coefficients."""
    return _blocks_op("cz_iwt_adjoint", blocks, wtype, stream)


def field_from_zfastest(arr, channel=0, stream=None):
    """hdf2cz's array layout -> the codec's field: arr is a CUDA tensor of
    shape (nx, ny, nz) or (nx, ny, nz, nch), z fastest, float32 or float64;
    returns a float32 (nz, ny, nx) field (x fastest)."""
    import torch
    assert arr.is_cuda and arr.is_contiguous() and arr.dtype in (torch.float32, torch.float64)
    nx, ny, nz = arr.shape[:3]
    nch = arr.shape[3] if arr.dim() == 4 else 1
    ctx = context(arr.device.index or 0)
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=arr.device)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(arr.device).cuda_stream
    ctx.check(ctx.L.cz_field_from_zfastest(ctx.h, C.c_void_p(arr.data_ptr()), arr.element_size(), nch, channel, nx,
                                           ny, nz, C.c_void_p(out.data_ptr()), C.c_void_p(st)))
    return out


def field_to_zfastest(field, out=None, channel=0, stream=None):
    """The codec's (nz, ny, nx) field -> cz2hdf's layout: channel `channel`
    of `out` (float32, shape (nx, ny, nz) or (nx, ny, nz, nch)), new if None."""
    import torch
    nz, ny, nx = field.shape
    if out is None:
        out = torch.empty((nx, ny, nz), dtype=torch.float32, device=field.device)
    nch = out.shape[3] if out.dim() == 4 else 1
    ctx = context(field.device.index or 0)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(field.device).cuda_stream
    ctx.check(ctx.L.cz_field_to_zfastest(ctx.h, C.c_void_p(field.data_ptr()), nx, ny, nz, nch, channel,
                                         C.c_void_p(out.data_ptr()), C.c_void_p(st)))
    return out


def diff_field(data, offsets, shape, reference, wtype=1, shuffle=False, encoder="lz4", blocks_per_chunk=1,
               file_bytes=None, out=None, stream=None):
    """Decompress and compare with `reference` (CUDA float32 field of the same
    shape) in one pass: cz2diff's statistics, and its RES line when the
    compressed size `file_bytes` is given."""
    import torch
    nz, ny, nx = shape
    dev = data.device
    ctx = context(dev.index or 0)
    prm = params(0.0, wtype, 0, shuffle, encoder, blocks_per_chunk)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    stats = (C.c_double * 9)()
    ctx.check(ctx.L.cz_field_diff(ctx.h, C.c_void_p(data.data_ptr()), C.c_void_p(offsets.data_ptr()),
                                  offsets.numel() - 1, nx, ny, nz, C.byref(prm), C.c_void_p(reference.data_ptr()),
                                  C.c_void_p(st), C.c_void_p(out.data_ptr() if out is not None else None), stats))
    keys = ["e_inf", "n_inf", "e_1", "n_1", "e_2", "n_2", "min", "max", "n"]
    res = dict(zip(keys, list(stats)))
    if file_bytes is not None:
        buf = C.create_string_buffer(256)
        ctx.check(ctx.L.cz_res_line(stats, int(file_bytes), buf, 256))
        res["res_line"] = buf.value.decode()
    return res


def res_line(stats, file_bytes):
    """cz2diff's RES line from statistics (dict as returned by diff_field)."""
    L = _lib.load()
    keys = ["e_inf", "n_inf", "e_1", "n_1", "e_2", "n_2", "min", "max", "n"]
    st = (C.c_double * 9)(*[float(stats[k]) for k in keys])
    buf = C.create_string_buffer(256)
    rc = L.cz_res_line(st, int(file_bytes), buf, 256)
    if rc != 0:
        raise CzError(rc, "cz_res_line failed")
    return buf.value.decode()


def decompress_field(data, offsets, shape, wtype=1, shuffle=False, encoder="lz4", blocks_per_chunk=1, out=None,
                     stream=None):
    """Decompress device chunks (uint8 tensor + int64 offsets tensor) into a
    CUDA field of the given (nz, ny, nx) shape."""
    import torch
    nz, ny, nx = shape
    dev = data.device
    ctx = context(dev.index or 0)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=dev)
    prm = params(0.0, wtype, 0, shuffle, encoder, blocks_per_chunk)
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    ctx.check(ctx.L.cz_field_decompress(ctx.h, C.c_void_p(data.data_ptr()), C.c_void_p(offsets.data_ptr()),
                                        offsets.numel() - 1, nx, ny, nz, C.byref(prm), C.c_void_p(st),
                                        C.c_void_p(out.data_ptr())))
    return out


def compress_to_image(field, eps, wtype=1, zerobits=0, shuffle=False, encoder="lz4", device=0, out=None):
    """Host field (numpy, (nz, ny, nx)) -> .cz image bytes, end to end. `out`
    may be a preallocated host uint8 buffer (pinned for full speed); the
    image is then returned as a view of it."""
    ctx = context(device)
    f = np.ascontiguousarray(field, np.float32)
    nz, ny, nx = f.shape
    prm = params(eps, wtype, zerobits, shuffle, encoder, 1)
    nblocks = (nx // 32) * (ny // 32) * (nz // 32)
    cap = nblocks * (4 + _lib.MAX_RECORD + 16) * 2 + 65536
    buf = out if out is not None else np.empty(cap, np.uint8)
    w = C.c_longlong(0)
    ctx.check(ctx.L.cz_compress_to_image(ctx.h, f.ctypes.data, nx, ny, nz, C.byref(prm), None, buf.ctypes.data,
                                         buf.size, C.byref(w)))
    return buf[: w.value]


def image_info(img):
    L = _lib.load()
    a = np.frombuffer(bytes(img), np.uint8)
    dims = (C.c_int * 3)()
    enc = C.c_int(-1)
    rc = L.cz_image_info(a.ctypes.data, a.size, dims, C.byref(enc))
    if rc != 0:
        raise CzError(rc, "not a .cz image")
    return (dims[2], dims[1], dims[0]), enc.value


def decompress_image(img, wtype=1, shuffle=False, device=0):
    """.cz image bytes -> host field (numpy, (nz, ny, nx))."""
    ctx = context(device)
    a = np.frombuffer(bytes(img), np.uint8)
    shape, _ = image_info(a)
    out = np.empty(shape, np.float32)
    ctx.check(ctx.L.cz_decompress_image(ctx.h, a.ctypes.data, a.size, int(wtype), 1 if shuffle else 0, None,
                                        out.ctypes.data, out.size))
    return out
