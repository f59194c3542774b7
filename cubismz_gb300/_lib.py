"""ctypes binding of libczgpu.so (C-ABI declared in include/czgpu.h).

The library is built in-tree (cubismz_gb300/build.py). There is no CPU
fallback: if the library is missing or no CUDA device is visible, calls
raise.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libczgpu.so")

CZ_OK = 0
CZ_E_ARG = -1
CZ_E_CUDA = -2
CZ_E_CORRUPT = -3
CZ_E_SPACE = -4
CZ_E_NOMEM = -5
ENCODER_NONE = 0
ENCODER_LZ4 = 1
ENCODER_ZLIB = 2

MASK_BYTES = 4096
BLOCK_ELEMS = 32768
MAX_RECORD = MASK_BYTES + 4 * BLOCK_ELEMS

# exported symbols, as declared in include/czgpu.h
EXPORTS = [
    "cz_create", "cz_destroy", "cz_last_error", "cz_set_timing", "cz_stage_times", "cz_set_lz4_effort",
    "cz_block_compress", "cz_block_decompress",
    "cz_lz4_bound", "cz_lz4_compress", "cz_lz4_decompress",
    "cz_field_compress", "cz_stream_copy", "cz_field_decompress", "cz_batch_compress",
    "cz_file_bytes", "cz_file_image", "cz_compress_to_image", "cz_image_info", "cz_decompress_image",
    "cz_blocks_compress_noalloc", "cz_iwt_linear", "cz_iwt_adjoint", "cz_refit",
    "cz_mini_bytes", "cz_mini_write", "cz_part_bytes", "cz_part_write", "cz_stream_part", "cz_tail_bytes",
    "cz_tail_write", "cz_plan_create", "cz_plan_launch", "cz_plan_result", "cz_plan_info", "cz_plan_last_error",
    "cz_plan_destroy", "cz_plan_shape", "cz_field_diff", "cz_res_line", "cz_field_from_zfastest", "cz_field_to_zfastest",
    "cz_zlib_decompress", "cz_zlib_bound", "cz_zlib_compress",
]
NOALLOC_MAX_BLOCKS = 16


class CzError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"czgpu error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("eps", C.c_float), ("wtype", C.c_int), ("zerobits", C.c_int), ("shuffle", C.c_int),
                ("encoder", C.c_int), ("blocks_per_chunk", C.c_int)]


class Stream(C.Structure):
    _fields_ = [("data", C.c_void_p), ("data_bytes", C.c_longlong), ("chunk_offsets", C.c_void_p),
                ("nchunks", C.c_int), ("nblocks", C.c_longlong), ("raw_bytes", C.c_longlong)]


_L = None


def load():
    """Load libczgpu.so (raises if it was not built)."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: run cubismz_gb300/build.py (python -m cubismz_gb300.build)")
    L = C.CDLL(LIB_PATH)
    vp, ip, fp, u8p = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_uint8)
    llp = C.POINTER(C.c_longlong)
    L.cz_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    L.cz_destroy.argtypes = [vp]
    L.cz_last_error.argtypes = [vp]
    L.cz_last_error.restype = C.c_char_p
    L.cz_set_timing.argtypes = [vp, C.c_int]
    L.cz_set_lz4_effort.argtypes = [vp, C.c_int]
    L.cz_stage_times.argtypes = [vp, fp, C.c_int]
    L.cz_block_compress.argtypes = [vp, fp, C.c_float, C.c_int, C.c_int, C.c_int, u8p, ip]
    L.cz_block_decompress.argtypes = [vp, u8p, C.c_int, C.c_int, C.c_int, fp]
    L.cz_lz4_bound.argtypes = [C.c_int]
    L.cz_lz4_compress.argtypes = [vp, u8p, C.c_int, u8p, C.c_int, ip]
    L.cz_lz4_decompress.argtypes = [vp, u8p, C.c_int, u8p, C.c_int, ip]
    L.cz_zlib_decompress.argtypes = [vp, u8p, C.c_int, u8p, C.c_int, ip]
    L.cz_zlib_bound.argtypes = [C.c_int]
    L.cz_zlib_compress.argtypes = [vp, u8p, C.c_int, u8p, C.c_int, ip]
    L.cz_field_compress.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(Params), vp, C.POINTER(Stream)]
    L.cz_stream_copy.argtypes = [vp, C.POINTER(Stream), vp, vp, vp]
    L.cz_field_decompress.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Params), vp, vp]
    L.cz_batch_compress.argtypes = [vp, C.c_int, C.POINTER(C.c_void_p), ip, fp, C.POINTER(Params), vp,
                                    C.POINTER(Stream)]
    L.cz_file_bytes.argtypes = [vp, C.POINTER(Stream), C.c_int, C.c_int, C.c_int, C.POINTER(Params)]
    L.cz_file_bytes.restype = C.c_longlong
    L.cz_file_image.argtypes = [vp, C.POINTER(Stream), C.c_int, C.c_int, C.c_int, C.POINTER(Params), vp,
                                C.c_longlong, llp]
    L.cz_compress_to_image.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(Params), vp, vp, C.c_longlong,
                                       llp]
    L.cz_image_info.argtypes = [vp, C.c_longlong, ip, ip]
    L.cz_decompress_image.argtypes = [vp, vp, C.c_longlong, C.c_int, C.c_int, vp, vp, C.c_longlong]
    L.cz_blocks_compress_noalloc.argtypes = [vp, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, vp, vp, vp]
    L.cz_iwt_linear.argtypes = [vp, vp, C.c_longlong, C.c_int, vp, vp]
    L.cz_iwt_adjoint.argtypes = [vp, vp, C.c_longlong, C.c_int, vp, vp]
    L.cz_refit.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(Params), C.c_int, vp, C.POINTER(Stream)]
    L.cz_mini_bytes.restype = C.c_longlong
    L.cz_mini_write.argtypes = [C.c_longlong, vp, C.c_longlong]
    L.cz_part_bytes.argtypes = [C.c_longlong, C.c_int]
    L.cz_part_bytes.restype = C.c_longlong
    L.cz_part_write.argtypes = [vp, llp, C.c_int, vp, C.c_longlong, llp]
    L.cz_stream_part.argtypes = [vp, C.POINTER(Stream), vp, C.c_longlong, llp]
    L.cz_plan_create.argtypes = [vp, C.c_int, C.POINTER(C.c_void_p), ip, fp, C.POINTER(Params), C.c_int,
                                 C.POINTER(C.c_void_p)]
    L.cz_plan_launch.argtypes = [vp, vp]
    L.cz_plan_result.argtypes = [vp, vp, C.POINTER(Stream), C.POINTER(Stream)]
    L.cz_plan_shape.argtypes = [vp, ip, fp]
    L.cz_plan_info.argtypes = [vp, ip, fp]
    L.cz_plan_last_error.argtypes = [vp]
    L.cz_plan_last_error.restype = C.c_char_p
    L.cz_plan_destroy.argtypes = [vp]
    L.cz_field_diff.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Params), vp, vp, vp,
                                C.POINTER(C.c_double)]
    L.cz_res_line.argtypes = [C.POINTER(C.c_double), C.c_longlong, C.c_char_p, C.c_int]
    L.cz_field_from_zfastest.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
    L.cz_field_to_zfastest.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
    L.cz_tail_bytes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Params)]
    L.cz_tail_bytes.restype = C.c_longlong
    L.cz_tail_write.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, llp, ip, C.POINTER(Params), vp, C.c_longlong,
                                llp]
    _L = L
    return L
