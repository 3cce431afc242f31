import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return load


@pytest.fixture
def tc_layout():
    """Run the tensor-core calls of a test with a fixed tile layout (1: 64 x 64
    tiles, 2: 64 x 128 tiles); the tuned configuration is restored after."""
    import contextlib

    @contextlib.contextmanager
    def use(layout):
        from pg_gpu_gb300 import _lib as L, autotune
        h = L.handle()
        saved = autotune.lookup
        autotune.lookup = lambda kind, words: (layout, 0)
        autotune._applied.pop(h, None)
        try:
            yield
        finally:
            autotune.lookup = saved
            autotune._applied.pop(h, None)
            L.check(L.lib().pgld_set_tc_config(h, 0, 0), h)
    return use
