import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")
    config.addinivalue_line("markers", "slow: long statistical run")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as o

    if not os.path.exists(o.ORACLE_SO):
        o.build_oracle(with_reference=False)
    return o


@pytest.fixture(scope="session")
def ref_available(oracle_mod):
    if not os.path.isdir(oracle_mod.REF_SRC):
        return False
    if not os.path.exists(oracle_mod.REF_SO):
        oracle_mod.build_oracle(with_reference=True)
    return os.path.exists(oracle_mod.REF_SO)


@pytest.fixture(scope="session")
def gpu_lib():
    import hsmc_gb300
    from hsmc_gb300 import _native, build

    if not os.path.exists(_native.LIB_PATH):
        build.build()
    return hsmc_gb300
