"""Shared fixtures: repository paths, the `gpu` marker, library loaders."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "fel-multi-phase-flow_gb300")
for p in (PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libfmf.so")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle


@pytest.fixture(scope="session")
def fmf_built():
    """Path of the built library (no GPU needed to load it or to call its host code)."""
    from fmf import build
    return build.build()


@pytest.fixture(scope="session")
def fmf_lib():
    """The CUDA library, built in-tree; a GPU test fails (not skips) when it is missing."""
    from fmf import build, capi
    build.build()
    return capi.load()
