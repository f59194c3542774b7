"""Build libczgpu.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object under
cubismz_gb300/_build/, then one shared library is linked next to this file.
Flags: --fmad=false keeps every binary32 multiply and add separately rounded
unless the code asks for an fma explicitly (the codec is bit-exact to the
reference), -lineinfo for profiling.

Usage: python -m cubismz_gb300.build [--force] [--verbose]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libczgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["cz_codec.cu", "cz_lz4.cu", "cz_stream.cu", "cz_api.cu", "cz_noalloc.cu", "cz_refit.cu", "cz_ingest.cu", "cz_zlib.cu", "cz_format.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "czgpu.h")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    deps = _deps()
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ, src + ".o")
        if not force and not _stale(obj, deps):
            return obj
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I" + INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
        if verbose and src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}{r.stderr}")
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        os.replace(obj + ".tmp", obj)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
