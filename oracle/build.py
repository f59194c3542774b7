"""Build recipe for the CPU oracle and, where the reference sources are
present, for the reference's own codec compiled from those sources.

TEST INFRASTRUCTURE ONLY: the outputs are checkers and the CPU baseline,
never part of the product path.

  oracle/_build/libczoracle.so       plain-C restatement (czoracle.c), OpenMP
  oracle/_ref/libczref_<variant>.so  reference WaveletCompressor.cpp + lz4.c +
                                     the writer/reader headers, one library per
                                     compile-time feature set of the reference
                                     (Tools/Makefile:60-93 macro matrix)

Usage: python oracle/build.py [--ref]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFOUT = os.path.join(HERE, "_ref")
REFROOT = os.environ.get("CZ_REFERENCE_ROOT", "/root/reference")

# zerobits x shuffle x encoder, as the reference selects them at compile time
REF_VARIANTS = {}
for zb in (0, 4):
    for sh in (0, 1):
        for enc in ("none", "lz4", "zlib"):
            name = f"zb{zb}_sh{sh}_{enc}"
            flags = []
            if zb:
                flags += ["-D_USE_ZEROBITS_", f"-D_ZEROBITS_={zb}"]
            if sh:
                flags += ["-D_USE_SHUFFLE3_"]
            if enc == "lz4":
                flags += ["-D_USE_LZ4_"]
            elif enc == "zlib":
                flags += ["-D_USE_ZLIB_"]
            REF_VARIANTS[name] = flags


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    """Compile the plain-C oracle. -ffp-contract=off keeps binary64 products
    and sums separately rounded on every host (GCC contracts to FMA by
    default on aarch64)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "czoracle.c")
    out = os.path.join(BUILD, "libczoracle.so")
    if force or _stale(out, [src, os.path.join(HERE, "czoracle.h")]):
        _run(["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
              "-fPIC", "-shared", "-o", out + ".tmp", src, "-lm"])
        os.replace(out + ".tmp", out)
    return out


def reference_available():
    return os.path.isfile(os.path.join(REFROOT, "Compressor", "source", "WaveletCompressor.cpp"))


def _zlib_available():
    return os.path.isfile("/usr/include/zlib.h")


def build_ref(force=False):
    """Compile the reference's own sources (read in place, never copied)
    into one shared library per feature variant. Needs the reference tree
    and zlib headers (always included by WaveletCompressor.h:21)."""
    if not reference_available() or not _zlib_available():
        return []
    os.makedirs(REFOUT, exist_ok=True)
    src = os.path.join(REFROOT, "Compressor", "source")
    cub = os.path.join(REFROOT, "Compressor", "Cubism", "source")
    lz4 = os.path.join(REFROOT, "ThirdParty", "lz4")
    stub = os.path.join(HERE, "refstub")
    lz4o = os.path.join(REFOUT, "lz4.o")
    if force or _stale(lz4o, [os.path.join(lz4, "lz4.c")]):
        _run(["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-c", "-o", lz4o, os.path.join(lz4, "lz4.c")])
    common = ["g++", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-w",
              "-D_FLOAT_PRECISION_", "-D_BLOCKSIZE_=32", "-D_USE_WAVZ_", "-DTOTAL_CHANNELS=1", "-DNDEBUG",
              "-I" + stub, "-I" + src, "-I" + cub, "-I" + lz4]
    deps = [os.path.join(stub, "ref_harness.cpp"), os.path.join(stub, "mpi.h"),
            os.path.join(src, "WaveletCompressor.cpp")]

    def one(item):
        name, flags = item
        out = os.path.join(REFOUT, f"libczref_{name}.so")
        if force or _stale(out, deps):
            _run(common + flags + ["-shared", "-o", out + ".tmp", os.path.join(stub, "ref_harness.cpp"),
                                   os.path.join(src, "WaveletCompressor.cpp"), lz4o, "-lz"])
            os.replace(out + ".tmp", out)
        return out

    with ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        return list(ex.map(one, REF_VARIANTS.items()))


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        for p in build_ref(force="--force" in sys.argv):
            print(p)
