"""Profiling case for the codec kernels: a 256x512x512 fp32 field (256 MiB,
larger than L2; 60 blobs, 6 interfaces, seed 3), compressed three times with
wtype 1, threshold 1e-3 x range, zerobits 4, shuffle and the chosen lossless
stage (LZ4 by default, or zlib), then decompressed twice. Prints the
per-stage device times of each call. With --ingest, the same field goes
through the HDF5 tools' layout instead: to z-fastest and back, three times
each (the tile transpose kernels). --shape nz,ny,nx picks another field
size (multiples of 32), e.g. 512,512,512 for the bench's occupancy;
--bench-field takes the bench's own 512^3 field. --refit runs the CGLS refit
path twice instead, on the 256^3 refit field (60 blobs, 6 interfaces, seed
0; absolute threshold 1e-3, 10 steps, wtype 1, zerobits 4, shuffle, LZ4).

    python -m cubismz_gb300.profile_case [--encoder lz4|zlib] [--ingest] [--refit] [--shape nz,ny,nx] [--bench-field]
"""
import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--encoder", default="lz4", choices=["lz4", "zlib"])
    ap.add_argument("--ingest", action="store_true")
    ap.add_argument("--refit", action="store_true")
    ap.add_argument("--shape", default="256,512,512")
    ap.add_argument("--bench-field", action="store_true",
                    help="the bench's 512^3 field (200 blobs, 12 interfaces, seed 0) instead")
    args = ap.parse_args()
    enc = args.encoder
    import torch
    import cubismz_gb300 as cz
    from cubismz_gb300 import synth
    shape = tuple(int(x) for x in args.shape.split(","))
    if args.refit:
        f = torch.from_numpy(synth.config_field("refit", 0)).cuda()
        for _ in range(2):
            cf = cz.refit_field(f, 1e-3, 10, 1, 4, True, encoder=enc)
        torch.cuda.synchronize()
        print("refit payload", cf.nbytes)
        return
    if args.bench_field:
        field = synth.config_field("large", 0)
        shape = field.shape
    else:
        field = synth.generate(shape, seed=3, blobs=60, interfaces=6)
    eps = float(np.float32(1e-3 * (field.max() - field.min())))
    f = torch.from_numpy(field).cuda()
    if args.ingest:
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        for _ in range(3):
            ev[0].record()
            z = cz.field_to_zfastest(f)
            ev[1].record()
            back = cz.field_from_zfastest(z)
            ev[2].record()
            torch.cuda.synchronize()
            assert torch.equal(back, f)
            print("to_zfastest ms", ev[0].elapsed_time(ev[1]), "from_zfastest ms", ev[1].elapsed_time(ev[2]))
        return
    ctx = cz.context(0)
    ctx.set_timing(True)
    for _ in range(3):
        cf = cz.compress_field(f, eps, 1, 4, True, encoder=enc)
        print(f"compress stages ms (encode, {enc}, assembly):", ctx.stage_times(), "raw", cf.raw_bytes,
              "payload", cf.nbytes)
    data, off = cf.to_device()
    for _ in range(2):
        cz.decompress_field(data, off, shape, 1, True, encoder=enc)
        print(f"decompress stages ms ({enc}, locate, decode):", ctx.stage_times())
    torch.cuda.synchronize()


if __name__ == "__main__":
    main()
