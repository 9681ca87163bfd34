import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("sih-26_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine on cuda:0)")


@pytest.fixture(scope="session")
def built():
    """Build the generators and the checker (and the reference checker where the reference
    tree exists). The CUDA library is built too: nvcc cross-compiles without a GPU."""
    from sankhya_gb300 import build
    import pyoracle

    build.build_lpgen()
    pyoracle.build(reference=True)
    build.build_engine()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    import pyoracle

    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference(built):
    import pyoracle

    if not pyoracle.reference_available():
        pytest.skip("the reference tree is not present here, so oracle/_ref is not built")
    return pyoracle.Oracle(reference=True)


@pytest.fixture(scope="session")
def engine(built):
    """A GPU engine on cuda:0. Fails (does not skip) when the library cannot run: a GPU test
    must never pass on a fallback."""
    from sankhya_gb300 import capi

    eng = capi.PdhgEngine(0)
    yield eng
    eng.close()
