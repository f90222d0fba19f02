"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and run the CUDA path through the C ABI;
everything else runs on the CPU (oracle pins, ingest, ABI surface, CLI parsing,
multi-process sharding over gloo)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ipdps-crs-cmp-code_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the CUDA path")


@pytest.fixture(scope="session")
def semb_lib():
    import semb
    semb.lib()
    return semb
