import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def afv():
    from afivo_gb300 import build
    build.build()
    import afivo_gb300
    return afivo_gb300


@pytest.fixture(scope="session")
def gpu(afv):
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so.13")
        n = ctypes.c_int(0)
        ok = rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        ok = False
    if not ok:
        try:
            import torch
            ok = torch.cuda.is_available()
        except Exception:
            ok = False
    if not ok:
        pytest.fail("no CUDA device visible for a test marked gpu")
    return afv
