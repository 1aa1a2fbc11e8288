import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    # GBCC_SIM_LIB: run the tests against the host simulation of the device
    # side (tests/harness/sim) instead of the CUDA library; set only by
    # tests/test_sim_glue.py for its child pytest runs
    sim = os.environ.get("GBCC_SIM_LIB")
    if sim:
        from sisi4s_gb300 import capi
        capi.load(sim)


@pytest.fixture(scope="session")
def ctx():
    from sisi4s_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()
