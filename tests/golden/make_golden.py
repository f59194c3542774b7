"""Generate the committed golden fixtures from the reference.

Run where the reference tree is available (it is read from
/root/reference, or $CZ_REFERENCE_ROOT):

    python tests/golden/make_golden.py

Outputs (in this directory):
  demo128_f32.xz     the demo.h5 field of Tests/Data/data.tar.xz as raw
                     float32, x fastest (z,y,x), lzma-compressed. The HDF5
                     payload is the contiguous [X][Y][Z] array that starts at
                     byte 2144 (filesize - 128^3*4); Tools/Test_IO_Compressed.h
                     :192-217 maps element (gx,gy,gz) to block data[z][y][x].
  golden.json        - the reference's published RES line for demo.h5,
                       wtype 3, threshold 5e-5, zlib
                       (Tests/Test1/cselab_ref_run_all.txt:12), and the same
                       line recomputed by the reference writer+reader built
                       from its sources (oracle/_ref) with the .cz size;
                     - sha256 of reference records (WaveletCompressor::compress)
                       for seeded blocks over wtype x zerobits x shuffle x eps;
                     - sha256 of reference-decoded blocks for the same records;
                     - sha256 of the reference's pre-LZ4 chunk bytes of the
                       small synthetic field and of their LZ4_compress output.
  ref_lz4_chunks.bin small LZ4 streams produced by the reference LZ4_compress
                     (length-prefixed), for the GPU decoder tests.
  lz4_cases.json     the reference LZ4_uncompress_unknownOutputSize
                     (lz4.c:802-905) on seeded inputs: random bytes, valid
                     reference streams at exact, short and generous output
                     capacities, and the same streams with bytes changed or
                     cut; per case its return value (output size, or minus
                     the input position of the error) and the output's
                     sha256. Regenerate alone with --lz4-cases.
"""
import hashlib
import io
import json
import lzma
import os
import tempfile
import sys
import tarfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import czoracle as O  # noqa: E402
from cubismz_gb300 import synth  # noqa: E402

REF = os.environ.get("CZ_REFERENCE_ROOT", "/root/reference")
PUBLISHED = "RES:       256.23 8.722263e-04 8.271610e-05 3.972721e-05 1.046102e-04 3.611734e-08       0.1249      78.2226"


def demo_field():
    with tarfile.open(os.path.join(REF, "Tests", "Data", "data.tar.xz"), "r:xz") as t:
        raw = t.extractfile("demo.h5").read()
    n = 128 ** 3
    arr = np.frombuffer(raw[len(raw) - 4 * n:], dtype="<f4").reshape(128, 128, 128)  # [gx][gy][gz]
    return np.ascontiguousarray(arr.transpose(2, 1, 0))  # [z][y][x]


def res_line(orig, dec, fsize):
    """cz2diff's RES line (Tools/cz2diff.cpp:116-261)."""
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


def seeded_blocks():
    rng = np.random.default_rng(2024)
    small = synth.config_field("small", 0)
    out = [small[:32, :32, :32].copy(), small[32:64, 64:96, 96:128].copy()]
    out.append((rng.standard_normal(32 ** 3) * 1e-3 + 1.0).astype(np.float32).reshape(32, 32, 32))
    out.append((rng.standard_normal(32 ** 3) * 10.0 ** rng.uniform(-6, 6, 32 ** 3)).astype(np.float32)
               .reshape(32, 32, 32))
    return out


CASES = [(wt, zb, sh, eps) for wt in (1, 2, 3) for (zb, sh) in ((0, 0), (4, 1)) for eps in (0.0, 1e-3)]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def lz4_cases():
    """Seeded LZ4 decoder cases, decoded by the reference's own decoder."""
    L = O.ref(4, 1, "lz4")
    rng = np.random.default_rng(77)
    small = synth.config_field("small", 0)
    raw, off = O.field_compress(small, 1e-2, 1, 4, 1, 0, 1)
    plain = [raw[off[3]:off[3] + 2000].tobytes(), bytes(3000), b"abc" * 700,
             rng.integers(0, 256, 500, np.uint8).tobytes(),
             b"".join(bytes(rng.integers(0, 256, int(rng.integers(1, 40)), np.uint8)) + bytes([int(rng.integers(0, 256))])
                      * int(rng.integers(4, 90)) for _ in range(30))]
    streams = [O.ref_lz4_compress(L, d).tobytes() for d in plain]
    cases = []

    def add(kind, data, cap, base=None, edits=None, cut=None):
        n, out = O.ref_lz4_decompress(L, data, cap)
        c = {"kind": kind, "cap": cap, "ref": int(n), "sha": sha(out.tobytes()) if n > 0 else ""}
        if base is None:
            c["hex"] = data.hex()
        else:
            c["base"] = base
            if edits:
                c["edits"] = edits
            if cut is not None:
                c["cut"] = cut
        cases.append(c)

    for i in range(60):
        add("junk", rng.integers(0, 256, int(rng.integers(1, 300)), np.uint8).tobytes(), 4096 if i % 2 else 64)
    for b, (z, d) in enumerate(zip(streams, plain)):
        for cap in (len(d), len(d) - 1, len(d) // 2, len(d) + 100):
            add("valid", z, cap, base=b)
        for _ in range(12):
            edits = [[int(rng.integers(0, len(z))), int(rng.integers(0, 256))] for _ in range(int(rng.integers(1, 3)))]
            m = bytearray(z)
            for pos, val in edits:
                m[pos] = val
            add("edited", bytes(m), len(d), base=b, edits=edits)
        for cut in sorted(set(int(x) for x in rng.integers(1, len(z), 6))):
            add("cut", z[:cut], len(d), base=b, cut=cut)
    return {"streams": [z.hex() for z in streams], "cases": cases}


def main():
    if not os.path.isdir(REF):
        sys.exit("reference tree not found")
    if sys.argv[1:] == ["--lz4-cases"]:
        with open(os.path.join(HERE, "lz4_cases.json"), "w") as f:
            json.dump(lz4_cases(), f)
        return
    with open(os.path.join(HERE, "lz4_cases.json"), "w") as f:
        json.dump(lz4_cases(), f)
    field = demo_field()
    with open(os.path.join(HERE, "demo128_f32.xz"), "wb") as f:
        f.write(lzma.compress(field.tobytes(), preset=9))
    gold = {"published_res": PUBLISHED}
    L = O.ref(0, 0, "zlib")
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "demo.cz")
        O.ref_write_cz(L, field, 5e-5, 3, path, 1, 1)
        dec = O.ref_read_cz(L, path, 3)
        size = os.path.getsize(path)
    gold["reference_rebuilt_res"] = res_line(field, dec, size)
    gold["reference_rebuilt_cz_bytes"] = size
    gold["reference_demo_decoded_sha256"] = sha(dec.tobytes())
    os.remove(path)

    blocks = seeded_blocks()
    gold["block_cases"] = []
    for wt, zb, sh, eps in CASES:
        Lv = O.ref(zb, sh, "none")
        recs, decs = [], []
        for b in blocks:
            r = O.ref_block_compress(Lv, b, eps, wt)
            recs.append(sha(r))
            decs.append(sha(O.ref_block_decompress(Lv, r, wt).tobytes()))
        gold["block_cases"].append({"wtype": wt, "zerobits": zb, "shuffle": sh, "eps": eps,
                                    "record_sha256": recs, "decoded_sha256": decs})

    # pre-LZ4 stream of the small synthetic field (one record per chunk) and
    # the reference LZ4_compress of a few chunks (threshold 1e-2)
    small = synth.config_field("small", 0)
    Lz = O.ref(4, 1, "lz4")
    raw, off = O.field_compress(small, 1e-3, 1, 4, 1, 0, 1)
    gold["small_field_raw_sha256"] = sha(raw)
    gold["small_field_raw_bytes"] = int(off[-1])
    buf = io.BytesIO()
    lz = []
    raw2, off2 = O.field_compress(small, 1e-2, 1, 4, 1, 0, 1)
    for c in (0, 21, 42):
        chunk = raw2[off2[c]:off2[c + 1]]
        z = O.ref_lz4_compress(Lz, chunk)
        lz.append({"chunk": c, "raw_sha256": sha(chunk), "raw_bytes": len(chunk), "lz4_bytes": len(z)})
        buf.write(np.int32(len(z)).tobytes())
        buf.write(np.int32(len(chunk)).tobytes())
        buf.write(z.tobytes())
    gold["ref_lz4_chunks"] = lz
    with open(os.path.join(HERE, "ref_lz4_chunks.bin"), "wb") as f:
        f.write(buf.getvalue())
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print(gold["reference_rebuilt_res"])


if __name__ == "__main__":
    main()
