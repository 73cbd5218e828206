"""Shared test setup: import paths, the gpu marker, helpers.

CPU tests (-m "not gpu") check the oracle against the reference's own
kernels (oracle/_ref, when built) and against the committed golden fixtures,
and the C-ABI's host logic.  GPU tests (-m gpu) call the CUDA library
through the C ABI and compare it with the oracle on the same inputs.
"""
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "clij-opencl-kernels_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

DTYPES = [np.uint8, np.int8, np.uint16, np.int16, np.float32]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


def random_image(rng, shape, dtype, binary=False, density=0.8):
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        a = (rng.standard_normal(shape) * 300).astype(np.float32)
    else:
        info = np.iinfo(dtype)
        a = rng.integers(info.min, int(info.max) + 1, size=shape).astype(dtype)
    if binary:
        a = (a * (rng.random(shape) < density)).astype(dtype)
    return a


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.port()
    return O
