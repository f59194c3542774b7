"""Several ranks writing one .cz file: z-slab shards, the size exchange over
torch.distributed (gloo, 2 ranks on the CPU), parts written at the
exclusive scan of their sizes. The file decodes to the same field as the
single-rank path (oracle decoder on the chunks the file's LUTs name, and
the reference reader when it was built here); with one rank and the
reference's chunking the file is the reference writer's byte for byte."""
import os
import socket
import tempfile

import numpy as np
import pytest

from oracle import czoracle as O
from tests.helpers import parse_cz


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, path, field, eps, encoder, bpc):
    import torch.distributed as dist
    from cubismz_gb300 import api, build, shard
    build.build()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        z0, z1 = shard.slab(field.shape[0], rank, world)
        raw, off = O.field_compress(field[z0:z1], eps, 1, 4, 1, encoder, bpc, 1)
        part, n = shard.part_from_host(raw[: off[-1]], off)
        prm = api.params(eps, 1, 4, True, "lz4" if encoder == 1 else "none", bpc)
        shard.write_file(path, part, n, field.shape, prm, rank, world)
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def lib():
    from cubismz_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.mark.parametrize("world,encoder,bpc", [(2, 1, 1), (2, 0, 3), (4, 1, 2)])
def test_ranks_write_one_file(lib, small_field, world, encoder, bpc):
    import torch.multiprocessing as mp
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "f.cz")
        mp.spawn(_rank_main, args=(world, _port(), path, small_field, eps, encoder, bpc), nprocs=world, join=True)
        img = open(path, "rb").read()
    info = parse_cz(img)
    assert info["blocks"] == (4, 4, 4) and info["subdomain"] == (4, 4, 4 // world)
    assert len(info["ranks"]) == world
    # chunks in rank order are the single-rank chunks of the whole field
    chunks = [c for r in info["ranks"] for c in r]
    raw, off = O.field_compress(small_field, eps, 1, 4, 1, 0, 1, 1)  # records, one per chunk
    blocks_per_rank = 64 // world
    want = []
    for r in range(world):
        for c0 in range(0, blocks_per_rank, bpc):
            g0 = r * blocks_per_rank + c0
            g1 = min(g0 + bpc, (r + 1) * blocks_per_rank)
            want.append(bytes(raw[off[g0]:off[g1]]))
    if encoder == 1:
        got = []
        for c, w in zip(chunks, want):
            n, out = O.lz4_decompress(np.frombuffer(c, np.uint8), len(w))
            got.append(out.tobytes()[:n])
        chunks = got
    assert chunks == want
    # metadata: rank-local chunk ids and sub ids, global block coordinates
    for r in range(world):
        for l in range(blocks_per_rank):
            m = info["meta"][r * blocks_per_rank + l]
            assert m == (l // bpc, l % bpc, l % 4, (l // 4) % 4, r * (4 // world) + l // 16)
    L = O.ref(4, 1, "lz4" if encoder == 1 else "none")
    if L is not None:
        with tempfile.NamedTemporaryFile(suffix=".cz") as t:
            t.write(img)
            t.flush()
            dec = O.ref_read_cz(L, t.name, 1)
        assert np.array_equal(dec, O.field_decompress(raw, off, small_field.shape, 1, 1))


def test_single_rank_file_is_the_reference_writers(lib, small_field):
    """One rank, encoder none, 15 records per chunk (the reference's ENTRIES
    with one OpenMP thread): byte-identical to the reference writer."""
    L = O.ref(4, 1, "none")
    if L is None:
        pytest.skip("reference build not available")
    from cubismz_gb300 import api, shard
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    raw, off = O.field_compress(small_field, eps, 1, 4, 1, 0, 15, 1)
    part, n = shard.part_from_host(raw[: off[-1]], off)
    with tempfile.TemporaryDirectory() as d:
        mine, theirs = os.path.join(d, "a.cz"), os.path.join(d, "b.cz")
        shard.write_file(mine, part, n, small_field.shape, api.params(eps, 1, 4, True, "none", 15))
        O.ref_write_cz(L, small_field, eps, 1, theirs, 1, 1)
        assert open(mine, "rb").read() == open(theirs, "rb").read()


def test_single_rank_lz4_file_is_the_reference_writers(lib, small_field):
    """Encoder lz4, 15 records per chunk, one thread: the file assembled
    from the oracle's LZ4 chunks equals the reference writer's byte for
    byte (the restated LZ4_compress gives the reference's bytes)."""
    L = O.ref(4, 1, "lz4")
    if L is None:
        pytest.skip("reference build not available")
    from cubismz_gb300 import api, shard
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    z, off = O.field_compress(small_field, eps, 1, 4, 1, 1, 15, 1)
    part, n = shard.part_from_host(z[: off[-1]], off)
    with tempfile.TemporaryDirectory() as d:
        mine, theirs = os.path.join(d, "a.cz"), os.path.join(d, "b.cz")
        shard.write_file(mine, part, n, small_field.shape, api.params(eps, 1, 4, True, "lz4", 15))
        O.ref_write_cz(L, small_field, eps, 1, theirs, 1, 1)
        assert open(mine, "rb").read() == open(theirs, "rb").read()


def test_single_rank_zlib_file_is_the_reference_writers(lib, demo_field):
    """Encoder zlib, 15 records per chunk, one thread: the file assembled
    from zlib chunks equals the reference writer's byte for byte."""
    L = O.ref(0, 0, "zlib")
    if L is None:
        pytest.skip("reference build not available")
    from cubismz_gb300 import api, shard
    from tests.helpers import zlib_chunks
    raw, off = O.field_compress(demo_field, 5e-5, 3, 0, 0, 0, 1)
    z = zlib_chunks(raw, off, 15, 64)
    offs = np.concatenate([[0], np.cumsum([len(c) for c in z])]).astype(np.int64)
    part, n = shard.part_from_host(np.frombuffer(b"".join(z), np.uint8), offs)
    with tempfile.TemporaryDirectory() as d:
        mine, theirs = os.path.join(d, "a.cz"), os.path.join(d, "b.cz")
        shard.write_file(mine, part, n, demo_field.shape, api.params(5e-5, 3, 0, False, "zlib", 15))
        O.ref_write_cz(L, demo_field, 5e-5, 3, theirs, 1, 1)
        assert open(mine, "rb").read() == open(theirs, "rb").read()


@pytest.mark.parametrize("world", [2, 4])
def test_in_memory_multi_rank_image(lib, small_field, world):
    """The multi-rank image of tests.helpers.multi_rank_image (the GPU
    reader's multi-rank test input) parses, and the reference reader decodes
    it to the oracle's field."""
    import ctypes as C
    from tests.helpers import multi_rank_image
    eps = float(np.float32(1e-3 * (small_field.max() - small_field.min())))
    img = multi_rank_image(small_field, eps, world)
    buf = np.frombuffer(img, np.uint8).copy()
    dims, enc = (C.c_int * 3)(), C.c_int(-1)
    assert lib.cz_image_info(C.c_void_p(buf.ctypes.data), len(img), dims, C.byref(enc)) == 0
    assert list(dims) == [small_field.shape[2], small_field.shape[1], small_field.shape[0]] and enc.value == 1
    L = O.ref(4, 1, "lz4")
    if L is None:
        pytest.skip("reference build not available")
    raw, roff = O.field_compress(small_field, eps, 1, 4, 1, 0, 1)
    want = O.field_decompress(raw, roff, small_field.shape, 1, 1)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.cz")
        with open(path, "wb") as f:
            f.write(img)
        got = O.ref_read_cz(L, path, 1)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))

