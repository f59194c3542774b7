"""Writes the GPU-made .cz fixtures that tests/test_gpu_written_images.py
reads with the reference's own reader on CPU.

Run on a machine with a GPU (it needs libczgpu.so and a CUDA device):

    python tests/golden/make_gpu_images.py

Input: the 128^3 synthetic field of the plain-method workload (seeded, 20
blobs, 3 interfaces; the same bits on every host), threshold 1e-2 of its
range, wtype 1, zero-bits 4, shuffle. Each image is written end to end by
cz_compress_to_image (host field in, .cz image out), once with
`Encoder: lz4` and once with `Encoder: zlib`:

    gpu_small_lz4.cz, gpu_small_zlib.cz

The GPU's LZ4 and DEFLATE bytes are its own (any reader of the format must
decode them), so the fixtures are remade whenever the encoders change.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

REL_THR, WTYPE, ZEROBITS, SHUFFLE = 1e-2, 1, 4, True


def field_and_eps():
    from cubismz_gb300 import synth
    f = synth.config_field("small", 0)
    return f, float(np.float32(REL_THR * float(f.max() - f.min())))


def main():
    import cubismz_gb300 as cz
    f, eps = field_and_eps()
    for enc in ("lz4", "zlib"):
        img = cz.compress_to_image(f, eps, WTYPE, ZEROBITS, SHUFFLE, encoder=enc)
        path = os.path.join(HERE, f"gpu_small_{enc}.cz")
        with open(path, "wb") as fh:
            fh.write(bytes(img))
        print(path, len(img))


if __name__ == "__main__":
    main()
