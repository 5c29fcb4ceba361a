"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


class _ArithLib:
    """The package with VPM handles created in one arithmetic ('fp64', the
    library default and the reference's, or 'ff48'); every other attribute
    is the package's own."""

    def __init__(self, mod, arith):
        self._mod = mod
        self.arith = arith

        class VPM(mod.VPM):
            def __init__(self, cfg, device=-1, arith=arith):
                super().__init__(cfg, device, arith)

        self.VPM = VPM

    def __getattr__(self, name):
        return getattr(self._mod, name)


@pytest.fixture(scope="session", params=["fp64", "ff48"])
def gpulib(request):
    """The library, once per arithmetic of the heavy kernels: every test
    that takes it runs in IEEE FP64 and in float-float."""
    import vpm_free_gb300 as V
    from vpm_free_gb300 import build
    build.build()
    return _ArithLib(V, request.param)

TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)
