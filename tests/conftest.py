import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "emulation: the kernels run on the CPU under a CUDA emulation "
                            "(one OS thread per CUDA thread, AddressSanitizer); opt in with CB_EMULATION=1")


def pytest_collection_modifyitems(config, items):
    """The emulation tests take tens of minutes on a few cores, so the default CPU suite
    leaves them out; CB_EMULATION=1 runs them."""
    if os.environ.get("CB_EMULATION") == "1":
        return
    skip = pytest.mark.skip(reason="CPU emulation of the kernels: set CB_EMULATION=1 to run")
    for it in items:
        if "emulation" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def cblib():
    """The built C-ABI library (built on demand)."""
    from cudabubble_gb300 import build, capi
    build.build()
    return capi.lib()
