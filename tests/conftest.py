"""Shared fixtures.  `gpu` marks tests that need a GB300 and libhp_cuda.so;
everything else runs on CPU (oracle, host logic, ABI symbol table)."""
import os
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc  # oracle/oracle.py
    orc.load()
    return orc


@pytest.fixture(scope="session")
def cpu(oracle):
    return oracle.CpuBackend()


@pytest.fixture(scope="session")
def native_lib():
    from hyperplonk_gb300 import build as b
    b.build()
    from hyperplonk_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def gpu(native_lib):
    from hyperplonk_gb300.backend import CudaBackend
    return CudaBackend(int(os.environ.get("HYPERPLONK_CUDA_TEST_DEVICE", "0")))


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = ROOT / "tests" / "golden"

    class G:
        fr = np.load(d / "fr_ops.npz")
        fq = np.load(d / "fq_ops.npz")
        wide = np.load(d / "wide_reduction.npz")
        g1 = np.load(d / "g1_ops.npz")
        msm = np.load(d / "msm.npz")
    return G
