import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libptn_gb300.so")


@pytest.fixture(autouse=True)
def _mixed_plans_at_every_size(monkeypatch):
    """The engine runs chains below DeviceNetwork.MIXED_MIN_FLOPS in FP64 even on
    the mixed path (a speed choice); the tests use small tensors and must still
    exercise the tensor-core plans, so the threshold is lifted here."""
    from pytreenet_gb300.engine import DeviceNetwork
    monkeypatch.setattr(DeviceNetwork, "MIXED_MIN_FLOPS", 0)
