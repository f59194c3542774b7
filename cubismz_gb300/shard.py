"""Several ranks, one .cz file: the collective layout of the reference writer
(SerializerIO_WaveletCompression_MPI_Simple.h:347-466) over
torch.distributed.

The grid is split into z-slabs, one per rank. Every rank compresses its slab
independently (no data-path collective) and forms its part -- its chunks and
the LUT of their offsets. The only exchange is each rank's part size and
chunk count (the writer's MPI_Exscan of sizes, :389, and the gather of the
HeaderLUT): part r goes at the mini header plus the sizes of parts 0..r-1,
rank 0 writes the mini header and the tail (header, BlockMetadata,
HeaderLUT) after the last part. Each rank writes with pwrite at its own
offset, like the reference's MPI-IO writes.

The layout functions run on the host (libczgpu.so, no GPU needed); the
exchange runs on any torch.distributed backend (gloo, nccl).
"""
import ctypes as C
import os

import numpy as np

from . import _lib


def slab(nz, rank, world):
    """Cell range [z0, z1) of rank's z-slab of a grid nz cells deep."""
    bz = nz // 32
    if nz % 32 or bz % world:
        raise ValueError(f"{bz} block layers do not split into {world} slabs")
    per = bz // world
    return 32 * per * rank, 32 * per * (rank + 1)


def part_from_host(payload, offsets):
    """A rank's part from chunks in host memory: payload bytes and chunk
    offsets (nchunks + 1, starting at 0)."""
    L = _lib.load()
    pay = np.ascontiguousarray(payload, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    n = len(off) - 1
    out = np.empty(L.cz_part_bytes(int(off[-1]), n), np.uint8)
    w = C.c_longlong(0)
    rc = L.cz_part_write(C.c_void_p(pay.ctypes.data), off.ctypes.data_as(C.POINTER(C.c_longlong)), n,
                         C.c_void_p(out.ctypes.data), out.size, C.byref(w))
    if rc != 0:
        raise _lib.CzError(rc, "cz_part_write failed")
    return out[: w.value], n


def part_from_stream(cf):
    """A rank's part from a compressed field held on its GPU."""
    L = cf.ctx.L
    out = np.empty(L.cz_part_bytes(cf.nbytes, cf.s.nchunks), np.uint8)
    w = C.c_longlong(0)
    cf.ctx.check(L.cz_stream_part(cf.ctx.h, C.byref(cf.s), C.c_void_p(out.ctypes.data), out.size, C.byref(w)))
    return out[: w.value], cf.s.nchunks


def _gather_sizes(part_bytes, nchunks, world, group):
    if world == 1:
        return [int(part_bytes)], [int(nchunks)]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    mine = torch.tensor([int(part_bytes), int(nchunks)], dtype=torch.int64, device=dev)
    alls = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(alls, mine, group=group)
    return [int(t[0]) for t in alls], [int(t[1]) for t in alls]


def write_file(path, part, nchunks, shape, prm, rank=0, world=1, group=None):
    """Write this rank's part of the .cz file at `path` (global field shape
    (nz, ny, nx), params `prm` from api.params); rank 0 also writes the mini
    header and the tail. Returns the file size."""
    L = _lib.load()
    nz, ny, nx = shape
    bx, by, bz = nx // 32, ny // 32, nz // 32
    sizes, chunks = _gather_sizes(len(part), nchunks, world, group)
    mini = L.cz_mini_bytes()
    tb = L.cz_tail_bytes(bx, by, bz, world, C.byref(prm))
    if tb < 0:
        raise ValueError("grid does not split into the ranks' z-slabs")
    offset = mini + sum(sizes[:rank])
    header_offset = mini + sum(sizes)
    if rank == 0:
        head = np.empty(mini, np.uint8)
        rc = L.cz_mini_write(header_offset, C.c_void_p(head.ctypes.data), mini)
        if rc != 0:
            raise _lib.CzError(rc, "cz_mini_write failed")
        tail = np.empty(tb, np.uint8)
        pb = (C.c_longlong * world)(*sizes)
        pc = (C.c_int * world)(*chunks)
        w = C.c_longlong(0)
        rc = L.cz_tail_write(bx, by, bz, world, pb, pc, C.byref(prm), C.c_void_p(tail.ctypes.data), tb, C.byref(w))
        if rc != 0:
            raise _lib.CzError(rc, "cz_tail_write failed")
        with open(path, "wb") as f:
            f.write(head.tobytes())
            f.seek(header_offset)
            f.write(tail[: w.value].tobytes())
    _barrier(world, group)
    fd = os.open(path, os.O_WRONLY)
    try:
        os.pwrite(fd, np.ascontiguousarray(part).tobytes(), offset)
    finally:
        os.close(fd)
    _barrier(world, group)
    return header_offset + tb


def _barrier(world, group):
    if world > 1:
        import torch.distributed as dist
        dist.barrier(group=group)
