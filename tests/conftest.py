import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import _util  # noqa: E402,F401  (puts the package and oracle dirs on sys.path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def port():
    import pyoracle
    pyoracle.build()
    return pyoracle.Port()


@pytest.fixture(scope="session")
def ref():
    """The reference's own CPU code; only where its checkout was available."""
    import pyoracle
    pyoracle.build()
    if not os.path.exists(pyoracle.REF_PATH):
        pytest.skip("reference library not built here (no reference checkout)")
    return pyoracle.Ref()


@pytest.fixture(scope="session")
def sphx_lib():
    """libsphx.so, built in-tree; loading needs no GPU."""
    import build_sphx
    build_sphx.build()
    import sphx
    sphx.lib()
    return sphx


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(_util.GOLDEN, name + ".npz")))
    return load
