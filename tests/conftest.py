import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests through the C-ABI")
    config.addinivalue_line("markers", "slow: longer statistical checks")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_cpu.npz"))


@pytest.fixture(scope="session")
def cuda():
    """cuda:0 with libvpmc.so loaded (built on first use)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vortexparticlemc_cuda_gb300._lib import LIB_PATH
    if not os.path.exists(LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)


def to_dev(a, dev):
    import numpy as np
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)
