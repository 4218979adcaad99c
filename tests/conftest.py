import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity against the oracle")


@pytest.fixture(scope="session")
def built():
    """Builds the oracle and the CUDA library once per session."""
    from oracle import build as obuild
    from semantic_icpslam_gb300 import build as pbuild
    import synth
    obuild.build()
    pbuild.build()
    synth.build()
    return True
