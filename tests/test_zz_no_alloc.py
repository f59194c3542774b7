"""cz_blocks_compress_noalloc: the allocation-free entry point for callers
that cannot call cudaMalloc (their device memory is all in their own pool,
or an allocation would synchronise the device under them). It must give
the same records as the allocating per-block entry point, call after call,
although every call reuses the library's one static scratch array.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import seeded_blocks, sha

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(gpu_lib, golden):
    import torch
    import cubismz_gb300 as cz
    from cubismz_gb300 import _lib

    L = _lib.load()
    rng = np.random.default_rng(77)
    seeded = seeded_blocks()
    blocks = seeded + [(rng.standard_normal((32, 32, 32)) * 0.01 + 2.0).astype(np.float32)]
    cases = {(c["wtype"], c["zerobits"], c["shuffle"], c["eps"]): c for c in golden["block_cases"]}
    # two calls in a row with different parameters and block counts: the
    # second must not see anything the first left in the shared scratch
    calls = [(blocks, 1e-3, 1, 4, True), (blocks[:3], 1e-3, 3, 0, False)]
    for stack, eps, wtype, zb, sh in calls:
        n = len(stack)
        d_blocks = torch.from_numpy(np.stack(stack)).cuda().contiguous()
        d_records = torch.zeros(n * _lib.MAX_RECORD, dtype=torch.uint8, device="cuda")
        d_nbytes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.cz_blocks_compress_noalloc(C.c_void_p(d_blocks.data_ptr()), n, C.c_float(eps), wtype, zb,
                                          1 if sh else 0, C.c_void_p(d_records.data_ptr()),
                                          C.c_void_p(d_nbytes.data_ptr()), C.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        recs = d_records.cpu().numpy().reshape(n, _lib.MAX_RECORD)
        sizes = d_nbytes.cpu().numpy()
        wc = cz.WaveletCompressor(zerobits=zb, shuffle=sh)
        for g, b in enumerate(stack):
            wc.uncompressed_data()[...] = b
            nb = wc.compress(eps, False, wtype)
            assert sizes[g] == nb
            assert np.array_equal(recs[g, :nb], wc.compressed_data()[:nb])
        # the reference's own records of the seeded blocks (committed hashes)
        want = cases[(wtype, zb, int(sh), eps)]["record_sha256"]
        for g in range(min(n, len(seeded))):
            assert sha(recs[g, :sizes[g]]) == want[g]


def test_noalloc_rejects_too_many_blocks(gpu_lib):
    import torch
    from cubismz_gb300 import _lib

    L = _lib.load()
    n = _lib.NOALLOC_MAX_BLOCKS + 1
    d_blocks = torch.zeros((n, 32, 32, 32), dtype=torch.float32, device="cuda")
    d_records = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_nbytes = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = L.cz_blocks_compress_noalloc(C.c_void_p(d_blocks.data_ptr()), n, C.c_float(0.0), 1, 0, 0,
                                      C.c_void_p(d_records.data_ptr()), C.c_void_p(d_nbytes.data_ptr()), None)
    assert rc == _lib.CZ_E_ARG


def test_noalloc_rejects_misaligned_pointers(gpu_lib):
    """Blocks are read as 16-byte vectors, records and sizes written as
    32-bit words: offset views are refused before anything is launched."""
    import torch
    from cubismz_gb300 import _lib

    L = _lib.load()
    d_blocks = torch.zeros((2, 32, 32, 32), dtype=torch.float32, device="cuda")
    d_records = torch.zeros(2 * _lib.MAX_RECORD + 16, dtype=torch.uint8, device="cuda")
    d_nbytes = torch.zeros(4, dtype=torch.int32, device="cuda")
    b, r, n = d_blocks.data_ptr(), d_records.data_ptr(), d_nbytes.data_ptr()
    for pb, pr, pn in ((b + 4, r, n), (b, r + 1, n), (b, r, n + 2)):
        rc = L.cz_blocks_compress_noalloc(C.c_void_p(pb), 1, C.c_float(0.0), 1, 0, 0, C.c_void_p(pr),
                                          C.c_void_p(pn), None)
        assert rc == _lib.CZ_E_ARG
    # the aligned call still works afterwards
    rc = L.cz_blocks_compress_noalloc(C.c_void_p(b), 2, C.c_float(0.0), 1, 0, 0, C.c_void_p(r), C.c_void_p(n), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert (d_nbytes[:2].cpu().numpy() == 4096 + 4 * 64).all()
