"""cubismz_gb300: GB300-native wavelet compression path of CubismZ.

The compute path is libczgpu.so (hand-written CUDA for sm_103a behind the C
ABI in include/czgpu.h); this package is its Python binding and mirrors the
reference compressor interface (see api.py).
"""
from .api import (Context, CompressedField, WaveletCompressor, batch_compress, compress_field, compress_to_image,
                  context,
                  decompress_field, decompress_image, diff_field, field_from_zfastest,
                  field_to_zfastest, image_info, iwt_adjoint, iwt_linear, lz4_compress,
                  lz4_decompress, params, Plan, refit_field, res_line,
                  zlib_compress, zlib_decompress)
from ._lib import CzError

__all__ = ["Context", "CompressedField", "WaveletCompressor", "batch_compress", "compress_field", "compress_to_image",
           "context",
           "decompress_field", "decompress_image", "diff_field", "field_from_zfastest",
           "field_to_zfastest", "image_info", "iwt_adjoint", "iwt_linear", "lz4_compress",
           "lz4_decompress", "params", "Plan", "refit_field", "res_line", "zlib_compress", "zlib_decompress", "CzError"]
