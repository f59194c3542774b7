"""The C-ABI boundary without a GPU: libczgpu.so builds and loads, exports
every entry point include/czgpu.h declares (and the binding's list matches
the header), host-only entry points work, and device entry points fail
with a status instead of crashing when no GPU is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from cubismz_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared():
    text = open(os.path.join(ROOT, "include", "czgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w \*]*?\b(cz_\w+)\s*\(", text, flags=re.M))


def test_every_declared_symbol_is_exported(lib):
    from cubismz_gb300 import _lib
    names = declared()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing
    assert set(_lib.EXPORTS) == names


def test_host_entry_points(lib):
    assert lib.cz_lz4_bound(1000) == 1000 + 1000 // 255 + 16
    assert lib.cz_mini_bytes() == 8 + len("\n==============START-BINARY-OCEAN==============\n")
    assert lib.cz_part_bytes(100, 3) == 124
    bad = np.zeros(16, np.uint8)
    dims = (C.c_int * 3)()
    assert lib.cz_image_info(C.c_void_p(bad.ctypes.data), 16, dims, None) != 0


def test_device_entry_points_fail_cleanly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.cz_create(0, C.byref(h))
    assert rc != 0


def test_noalloc_pointer_checks_precede_any_cuda_call(lib):
    """cz_blocks_compress_noalloc refuses misaligned or NULL pointers and
    block counts beyond CZ_NOALLOC_MAX_BLOCKS with CZ_E_ARG before it touches
    the device (these addresses are never dereferenced)."""
    from cubismz_gb300 import _lib
    f = lib.cz_blocks_compress_noalloc
    ok_b, ok_r, ok_n = 0x10000, 0x20000, 0x30000
    for b, r, n in ((ok_b + 4, ok_r, ok_n), (ok_b + 8, ok_r, ok_n), (ok_b, ok_r + 1, ok_n), (ok_b, ok_r, ok_n + 2),
                    (0, ok_r, ok_n), (ok_b, 0, ok_n), (ok_b, ok_r, 0)):
        assert f(C.c_void_p(b), 1, C.c_float(0.0), 1, 0, 0, C.c_void_p(r), C.c_void_p(n), None) == _lib.CZ_E_ARG
    for nb in (0, -1, _lib.NOALLOC_MAX_BLOCKS + 1):
        assert f(C.c_void_p(ok_b), nb, C.c_float(0.0), 1, 0, 0, C.c_void_p(ok_r), C.c_void_p(ok_n),
                 None) == _lib.CZ_E_ARG


def test_lz4_effort_needs_a_context(lib):
    """cz_set_lz4_effort checks its arguments before anything else: a NULL
    context is refused with CZ_E_ARG whatever the level."""
    from cubismz_gb300 import _lib
    for level in (-1, 0, 1, 2, 3):
        assert lib.cz_set_lz4_effort(None, level) == _lib.CZ_E_ARG
