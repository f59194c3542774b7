"""cz2diff's RES line from the library's host formatter (cz_res_line):
statistics of the oracle's decode of demo.h5 give the published line."""
import numpy as np

from oracle import czoracle as O
from tests.helpers import cz_size, header_text, zlib_chunks


def stats_f64(orig, dec):
    """cz2diff's accumulators (Tools/cz2diff.cpp:116-160), binary64."""
    f1 = dec.astype(np.float64).ravel()
    f2 = orig.astype(np.float64).ravel()
    e = np.abs(f1 - f2)
    return {"e_inf": e.max(), "n_inf": np.abs(f2).max(), "e_1": e.sum(), "n_1": np.abs(f2).sum(),
            "e_2": (e * e).sum(), "n_2": (f2 * f2).sum(), "min": f2.min(), "max": f2.max(), "n": float(f2.size)}


def test_res_line_reproduces_published_golden(golden, demo_field):
    from cubismz_gb300 import build
    build.build()
    import cubismz_gb300 as cz
    raw, off = O.field_compress(demo_field, 5e-5, 3, 0, 0, 0, 1)
    z = zlib_chunks(raw, off, 15, 64)
    size = cz_size([len(c) for c in z], 64, header_text(4, 4, 4, 5e-5, "AverageInterpWavelet3rdOrder", "zlib"))
    dec = O.field_decompress(raw, off, demo_field.shape, 3)
    assert cz.res_line(stats_f64(demo_field, dec), size) == golden["published_res"]
