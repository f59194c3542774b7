"""The region-parallel LZ4 kernels (cubismz_gb300/csrc/cz_lz4rec.cu), their
exact source compiled for the host on a warp emulator (tests/emu/), with
AddressSanitizer where the compiler has it: on block-record chunks made by
the oracle, every chunk's LZ4 block decodes with the restated reference
decoder (LZ4_uncompress_unknownOutputSize, lz4.c:802-905) to its records,
no access leaves its buffer, and with one record per chunk the compressed
size stays within 1.5 % of the reference's own LZ4_compress on the same
chunks. Shuffled and plain
payloads, blocks that keep every coefficient (the largest records), several
records per chunk, and varying lane orders (same-address stores landing in
different orders, as on the GPU) are covered."""
import os
import subprocess

import numpy as np
import pytest

from oracle import czoracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
EMU = os.path.join(HERE, "emu")
KERNEL = os.path.join(HERE, "..", "cubismz_gb300", "csrc", "cz_lz4rec.cu")


@pytest.fixture(scope="module")
def emu_exe():
    out = os.path.join(EMU, "_build")
    os.makedirs(out, exist_ok=True)
    inc = os.path.join(out, "lz4rec_src.inc")
    exe = os.path.join(out, "lz4rec_emu")
    srcs = [KERNEL] + [os.path.join(EMU, f) for f in ("warp_emu.h", "lz4rec_emu.cpp", "lz4rec_main.cpp")]
    if not os.path.exists(exe) or any(os.path.getmtime(p) > os.path.getmtime(exe) for p in srcs):
        text = open(KERNEL).read()
        text = text.replace('#include "cz_codec.h"\n', "").replace('#include "cz_device.cuh"\n', "")
        text = text.replace("extern __shared__ __align__(16) unsigned char lzr_smem[];",
                            "unsigned char *lzr_smem = g_emu_smem;")
        with open(inc, "w") as f:
            f.write(text)
        base = ["g++", "-std=c++20", "-O1", "-g", "-I", out, "-I", EMU, "-o", exe,
                os.path.join(EMU, "lz4rec_main.cpp")]
        r = subprocess.run(base[:4] + ["-fsanitize=address", "-fno-omit-frame-pointer"] + base[4:],
                           capture_output=True, text=True)
        if r.returncode != 0:  # no AddressSanitizer here: plain build
            subprocess.check_call(base)
    return exe


def chunk_layout(raw, off, bpc, nblocks):
    """in_off/in_len per chunk and, per block, its record size and where its
    [int32 nbytes][record] starts (records back to back in each chunk)."""
    nch = len(off) - 1
    rec = np.zeros(nblocks, np.int32)
    dst = np.zeros(nblocks, np.int64)
    g = 0
    for c in range(nch):
        p = int(off[c])
        while p < off[c + 1]:
            nb = int(np.frombuffer(raw[p:p + 4].tobytes(), "<i4")[0])
            rec[g], dst[g] = nb, p
            p += 4 + nb
            g += 1
    assert g == nblocks
    return off[:-1].astype(np.int64), np.diff(off).astype(np.int32), rec, dst


def run_emu(exe, tmp, raw, off, bpc, shuffle, nblocks, seed, ctas=2):
    in_off, in_len, rec, dst = chunk_layout(raw, off, bpc, nblocks)
    with open(os.path.join(tmp, "in.bin"), "wb") as f:
        f.write(raw.tobytes())
    hdr = np.array([len(in_len), bpc, 1 if shuffle else 0, ctas, seed, 1 if bpc > 1 else 0], np.int32)
    with open(os.path.join(tmp, "meta.bin"), "wb") as f:
        f.write(hdr.tobytes() + np.int64(nblocks).tobytes() + in_off.tobytes() + in_len.tobytes() + rec.tobytes()
                + (dst.tobytes() if bpc > 1 else b""))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([exe, tmp], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "ERROR: AddressSanitizer" not in r.stderr
    out = np.fromfile(os.path.join(tmp, "out.bin"), np.uint8)
    doff = np.fromfile(os.path.join(tmp, "off.bin"), np.int64)
    return out, doff


CASES = {
    # name: (field slice, eps (relative to range; None: keep all), zerobits,
    #        shuffle, records per chunk, lane-order seeds, size bound vs the reference)
    "shuffled": (slice(0, 128), 1e-3, 4, True, 1, (1, 7), 1.015),
    "plain_payload": (slice(0, 32), 1e-3, 0, False, 1, (3,), 1.015),
    "all_kept": (slice(0, 32), None, 0, True, 1, (5,), 1.015),
    # several records per chunk: matches are searched within each record's
    # regions only (the reference also matches across records)
    "three_per_chunk": (slice(0, 32), 1e-3, 4, True, 3, (2,), 1.10),
    "fifteen_per_chunk": (slice(0, 64), 1e-2, 4, True, 15, (4,), 1.10),
}


@pytest.mark.parametrize("name", list(CASES))
def test_region_lz4_decodes_and_compresses(emu_exe, small_field, tmp_path, name):
    sl, rel, zb, sh, bpc, seeds, bound = CASES[name]
    field = np.ascontiguousarray(small_field[sl])
    eps = -1.0 if rel is None else float(np.float32(rel * (small_field.max() - small_field.min())))
    raw, off = O.field_compress(field, eps, 1, zb, 1 if sh else 0, 0, bpc)
    nblocks = field.size // 32 ** 3
    for seed in seeds:
        out, doff = run_emu(emu_exe, str(tmp_path), raw, off, bpc, sh, nblocks, seed)
        ours = ref = 0
        for c in range(len(off) - 1):
            want = raw[off[c]:off[c + 1]]
            n, dec = O.lz4_decompress(out[doff[c]:doff[c + 1]], len(want))
            assert n == len(want) and np.array_equal(dec, want), (name, seed, c)
            ours += int(doff[c + 1] - doff[c])
            ref += len(O.lz4_compress(want))
        assert ours <= bound * ref, (name, ours, ref)
