"""Shared test setup: the `gpu` marker, repository import path, fixtures."""
import json
import lzma
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libczgpu.so")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def demo_field():
    with open(os.path.join(GOLDEN, "demo128_f32.xz"), "rb") as f:
        return np.frombuffer(lzma.decompress(f.read()), np.float32).reshape(128, 128, 128).copy()


@pytest.fixture(scope="session")
def small_field():
    from cubismz_gb300 import synth
    return synth.config_field("small", 0)


@pytest.fixture(scope="session")
def gpu_lib():
    """libczgpu.so built in-tree; GPU tests fail loudly if it cannot load."""
    from cubismz_gb300 import build
    build.build()
    from cubismz_gb300 import _lib
    return _lib.load()
