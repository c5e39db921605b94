import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def pytest_collection_modifyitems(config, items):
    # GPU tests must never silently pass on a CPU machine: without a device they are skipped
    # only when the run did not select them explicitly with -m gpu.
    has_gpu = cuda_device_count() > 0
    if has_gpu:
        return
    selected_gpu = "gpu" in (config.getoption("-m") or "") and "not gpu" not in (config.getoption("-m") or "")
    if selected_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def cuda_device_count():
    """Number of CUDA devices via the driver API (no torch import needed)."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return 0
    if cu.cuInit(0) != 0:
        return 0
    n = ctypes.c_int()
    if cu.cuDeviceGetCount(ctypes.byref(n)) != 0:
        return 0
    return n.value


def rel_err(a, b, axis=None):
    """max |a - b| / max |b| (per slice along `axis` when given)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if axis is None:
        scale = np.abs(b).max()
        return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())
    a = np.moveaxis(a, axis, 0).reshape(a.shape[axis], -1)
    b = np.moveaxis(b, axis, 0).reshape(b.shape[axis], -1)
    out = []
    for x, y in zip(a, b):
        s = np.abs(y).max()
        out.append(float(np.abs(x - y).max() / s) if s > 0 else float(np.abs(x - y).max()))
    return max(out)
