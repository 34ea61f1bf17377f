import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "soverign-gpu-accelerator-_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _cuda_available():
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        try:
            import torch
            return torch.cuda.is_available()
        except Exception:
            return False


@pytest.fixture(scope="session")
def sk():
    import sankhya_gb300
    if not os.path.exists(sankhya_gb300.LIB_PATH):
        import build as pkg_build
        pkg_build.build()
    return sankhya_gb300


@pytest.fixture(scope="session")
def oracle():
    import sk_oracle
    if not os.path.exists(sk_oracle.ORACLE_LIB):
        sk_oracle.build()
    return sk_oracle


@pytest.fixture(scope="session")
def gpu(sk):
    if not _cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sk
