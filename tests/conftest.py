import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    from mcmc_for_ammsb_gb300 import build
    build.build()
    from mcmc_for_ammsb_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def small_net(native_lib):
    from mcmc_for_ammsb_gb300 import workloads
    net, opts = workloads.build("small")
    return net, opts
