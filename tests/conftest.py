import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "gpu-montecarlo-risk_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import mc_oracle
    mc_oracle.build()
    return mc_oracle


@pytest.fixture(scope="session")
def engine():
    """The engine library, built if needed (fails loudly if it cannot be)."""
    from riskgpu import build as b
    b.build()
    import riskgpu
    riskgpu.lib()
    return riskgpu


@pytest.fixture(scope="session")
def gpu(engine):
    if engine.lib().rg_device_count() < 1:
        pytest.fail("a GPU test ran where no CUDA device is visible")
    import torch
    torch.cuda.init()
    return engine
