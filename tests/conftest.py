"""pytest configuration: puts the repository root and tests/ on sys.path and
registers the ``gpu`` marker (tests that need a GB300 and the built library)."""
import os
import sys

_TESTS = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_TESTS)
for _p in (_ROOT, _TESTS):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfmod.so")
