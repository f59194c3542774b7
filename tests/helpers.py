"""Helpers shared by the tests (fixtures, block iteration, the RES line)."""
import hashlib
import zlib

import numpy as np


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def blocks(field):
    nz, ny, nx = field.shape
    for bz in range(nz // 32):
        for by in range(ny // 32):
            for bx in range(nx // 32):
                yield field[bz * 32:bz * 32 + 32, by * 32:by * 32 + 32, bx * 32:bx * 32 + 32].copy()


def seeded_blocks():
    """The blocks make_golden.py hashed the reference outputs of."""
    from cubismz_gb300 import synth
    rng = np.random.default_rng(2024)
    small = synth.config_field("small", 0)
    out = [small[:32, :32, :32].copy(), small[32:64, 64:96, 96:128].copy()]
    out.append((rng.standard_normal(32 ** 3) * 1e-3 + 1.0).astype(np.float32).reshape(32, 32, 32))
    out.append((rng.standard_normal(32 ** 3) * 10.0 ** rng.uniform(-6, 6, 32 ** 3)).astype(np.float32)
               .reshape(32, 32, 32))
    return out


def res_line(orig, dec, fsize):
    """cz2diff's RES line (Tools/cz2diff.cpp:116-261): CR, relative and mean
    errors, bits per sample and PSNR = 20 log10((max-min)/(2 sqrt(MSE)))."""
    f1 = dec.astype(np.float64).ravel()
    f2 = orig.astype(np.float64).ravel()
    err = np.abs(f1 - f2)
    n = f1.size
    e_inf, n_inf = err.max(), np.abs(f2).max()
    e1, n1 = err.sum(), np.abs(f2).sum()
    e2, n2 = (err * err).sum(), (f2 * f2).sum()
    mse = e2 / n
    psnr = 20 * np.log10((f2.max() - f2.min()) / (2 * np.sqrt(mse)))
    return "RES: %12.2f %.6e %.6e %.6e %.6e %.6e %12.04f %12.04f" % (
        4.0 * n / fsize, e_inf / n_inf, e1 / n1, e1 / n, np.sqrt(e2) / np.sqrt(n2), np.sqrt(e2) / n,
        fsize * 8.0 / n, psnr)


def header_text(bx, by, bz, threshold, wavelets, encoder):
    """The .cz ASCII header (SerializerIO_WaveletCompression_MPI_Simple.h:495-556)."""
    mx = max(bx, by, bz)
    h = (1.0 / mx) / 32

    def g(v):  # iostream default formatting: %g, precision 6
        return "%g" % v

    return ("\n==============START-ASCI-HEADER==============\n"
            "Endianess: little\nsizeofReal: 4\nsizeofsize_t: 8\nsizeofBlockMetadata: 20\n"
            "sizeofHeaderLUT: 12\nsizeofCompressedBlock: 20\nBlocksize: 32\n"
            f"Blocks: {bx} x {by} x {bz}\nExtent: {g(h * bx * 32)} {g(h * by * 32)} {g(h * bz * 32)}\n"
            f"SubdomainBlocks: {bx} x {by} x {bz}\nHalfFloat: no\nWavelets: {wavelets}\n"
            f"WaveletThreshold: {g(float(np.float32(threshold)))}\nEncoder: {encoder}\n"
            "==============START-BINARY-METABLOCKS==============\n")


OCEAN = "\n==============START-BINARY-OCEAN==============\n"
LUTTITLE = "\n==============START-BINARY-LUT==============\n"


def cz_size(chunk_sizes, nblocks, header):
    return 8 + len(OCEAN) + sum(chunk_sizes) + 8 * len(chunk_sizes) + len(header) + 20 * nblocks + len(LUTTITLE) + 12


def zlib_chunks(raw, off, bpc, nblocks):
    """Regroup one-record chunks into bpc-record chunks and deflate each with
    zlib's default level, as deflate_inplace does (CompressionEncoders.h:116-190)."""
    out = []
    for c0 in range(0, nblocks, bpc):
        c1 = min(nblocks, c0 + bpc)
        out.append(zlib.compress(bytes(raw[off[c0]:off[c1]]), 6))
    return out


def _lz4_len(out, n):
    """LZ4 length continuation bytes for n >= 15 (n - 15 as 255s and a rest)."""
    n -= 15
    while n >= 255:
        out.append(255)
        n -= 255
    out.append(n)


def lz4_random_stream(rng, nseq, final_lit=12):
    """A valid LZ4 block built sequence by sequence, and its decoded bytes.

    Literal and match lengths mix the common short ones with lengths that
    need continuation bytes (a few long enough to need more than eight),
    offsets mix 1..8 (overlapping, byte-periodic copies), distances inside
    a 128-byte input window and far ones; the last literal run is at least
    12 bytes, so the stream is accepted with an output capacity equal to
    its decoded size."""
    z = bytearray()
    out = bytearray()
    for i in range(nseq):
        r = rng.random()
        lit = int(rng.integers(0, 4)) if r < 0.7 else int(rng.integers(14, 40)) if r < 0.93 else \
            int(rng.integers(250, 700)) if r < 0.99 else int(rng.integers(2100, 5000))
        if not out and lit == 0:
            lit = 1
        r = rng.random()
        ml = int(rng.integers(4, 9)) if r < 0.7 else int(rng.integers(15, 40)) if r < 0.93 else \
            int(rng.integers(250, 700)) if r < 0.99 else int(rng.integers(2100, 5000))
        lits = rng.integers(0, 256, lit, np.uint8).tobytes()
        have = len(out) + lit
        r = rng.random()
        off = int(rng.integers(1, 9)) if r < 0.3 else int(rng.integers(9, 200)) if r < 0.7 else \
            int(rng.integers(200, 65536))
        off = max(1, min(off, have, 65535))
        tok = (min(lit, 15) << 4) | min(ml - 4, 15)
        z.append(tok)
        if lit >= 15:
            _lz4_len(z, lit)
        z += lits
        z += bytes((off & 255, off >> 8))
        if ml - 4 >= 15:
            _lz4_len(z, ml - 4)
        out += lits
        for k in range(ml):
            out.append(out[len(out) - off])
    lit = final_lit + int(rng.integers(0, 40))
    lits = rng.integers(0, 256, lit, np.uint8).tobytes()
    z.append(min(lit, 15) << 4)
    if lit >= 15:
        _lz4_len(z, lit)
    z += lits
    out += lits
    return bytes(z), bytes(out)


def parse_cz(img):
    """A .cz image read the way the reference reader reads it
    (Reader_WaveletCompression.h:255-560): header keys, BlockMetadata, and
    for every subdomain its chunks as named by its LUT."""
    hoff = int(np.frombuffer(img[:8], np.uint64)[0])
    text_end = img.index(b"==============START-BINARY-METABLOCKS==============\n", hoff)
    keys = {}
    for line in img[hoff:text_end].decode().splitlines():
        if ":" in line:
            k, v = line.split(":", 1)
            keys[k.strip()] = v.strip()
    dims = tuple(int(x) for x in keys["Blocks"].split(" x "))
    sub = tuple(int(x) for x in keys["SubdomainBlocks"].split(" x "))
    nblocks = dims[0] * dims[1] * dims[2]
    pos = text_end + len("==============START-BINARY-METABLOCKS==============\n")
    meta = [tuple(int(v) for v in np.frombuffer(img[pos + 20 * i:pos + 20 * i + 20], np.int32))
            for i in range(nblocks)]
    pos += 20 * nblocks
    pos += len(LUTTITLE)
    nsub = nblocks // (sub[0] * sub[1] * sub[2])
    base = 8 + len(OCEAN)
    ranks = []
    for s in range(nsub):
        agg = int(np.frombuffer(img[pos + 12 * s:pos + 12 * s + 8], np.uint64)[0])
        nch = int(np.frombuffer(img[pos + 12 * s + 8:pos + 12 * s + 12], np.int32)[0])
        lut = np.frombuffer(img[base + agg - 8 * nch:base + agg], np.uint64).astype(np.int64)
        ends = list(lut[1:]) + [agg - 8 * nch]
        ranks.append([img[base + a:base + b] for a, b in zip(lut, ends)])
        base += agg
    assert base == hoff
    return {"blocks": dims, "subdomain": sub, "meta": meta, "ranks": ranks, "keys": keys}


def lz4_cases():
    """The reference LZ4 decoder's results on seeded inputs
    (tests/golden/lz4_cases.json, made by tests/golden/make_golden.py):
    yields (input bytes, output capacity, reference return value, sha256 of
    the reference's output or "")."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "lz4_cases.json")) as f:
        d = json.load(f)
    streams = [bytes.fromhex(h) for h in d["streams"]]
    for c in d["cases"]:
        if "hex" in c:
            data = bytes.fromhex(c["hex"])
        else:
            data = bytearray(streams[c["base"]])
            for pos, val in c.get("edits", []):
                data[pos] = val
            if "cut" in c:
                data = data[: c["cut"]]
            data = bytes(data)
        yield data, c["cap"], c["ref"], c["sha"]


def multi_rank_image(field, eps, world):
    """A .cz image of `field` as `world` ranks write it (z-slabs, the
    oracle's LZ4 chunks of one record, each rank's part, then the tail),
    assembled in memory by the host writer functions."""
    import ctypes as C
    from oracle import czoracle as O
    from cubismz_gb300 import _lib, api, shard
    L = _lib.load()
    nz, ny, nx = field.shape
    parts, chunks = [], []
    for r in range(world):
        z0, z1 = shard.slab(nz, r, world)
        payload, off = O.field_compress(np.ascontiguousarray(field[z0:z1]), eps, 1, 4, 1, 1, 1)
        part, n = shard.part_from_host(payload[: off[-1]], off)
        parts.append(part.tobytes())
        chunks.append(n)
    prm = api.params(eps, 1, 4, True, "lz4", 1)
    mini = L.cz_mini_bytes()
    hoff = mini + sum(len(p) for p in parts)
    head = np.empty(mini, np.uint8)
    assert L.cz_mini_write(hoff, C.c_void_p(head.ctypes.data), mini) == 0
    tb = L.cz_tail_bytes(nx // 32, ny // 32, nz // 32, world, C.byref(prm))
    tail = np.empty(tb, np.uint8)
    w = C.c_longlong(0)
    assert L.cz_tail_write(nx // 32, ny // 32, nz // 32, world, (C.c_longlong * world)(*[len(p) for p in parts]),
                           (C.c_int * world)(*chunks), C.byref(prm), C.c_void_p(tail.ctypes.data), tb, C.byref(w)) == 0
    return head.tobytes() + b"".join(parts) + tail[: w.value].tobytes()

