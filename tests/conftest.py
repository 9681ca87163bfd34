import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The checker libraries (the oracle and the reference) run A^T y in an OpenMP parallel region
# every iteration. On the tests' small LPs a team wider than the free cores waits at every
# barrier for a descheduled thread, and a solve of 1e6 iterations then takes tens of minutes
# on a busy machine. Their results do not depend on the team size (each column's sum is
# serial), so the tests run them on one thread unless the caller says otherwise. The bench's
# CPU legs set their own thread counts.
os.environ.setdefault("OMP_NUM_THREADS", "1")
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


def _reference_tree():
    """The reference checkout, else its staged copy (oracle/_ref/stage), else the checkout's
    expected path (where the tests that need it skip)."""
    import pyoracle

    return pyoracle.reference_tree() or pyoracle.REFERENCE_TREE


def core_link_args():
    """Compiler arguments for the reference's whole core (oracle/_ref/libsankhya_core.a, built
    by `make -C oracle ref-core` as a CUDA build compiles it), the four seam files in place of
    src/gpu, the C-ABI stand-in (tests/host/seam_standin.cpp) and the checkpoint stub. Skips
    the calling test where the reference tree or g++ is absent."""
    import shutil
    import subprocess

    ref = _reference_tree()
    if not os.path.isdir(os.path.join(ref, "src", "gpu")) or shutil.which("g++") is None:
        pytest.skip("the reference tree (or g++) is not present here")
    import torch

    subprocess.run(["make", "-s", f"-j{os.cpu_count() or 4}", "-C",
                    os.path.join(ROOT, "oracle"), "ref-core", f"REF={ref}"], check=True)
    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    flags = ["-std=c++20", "-O1", "-fPIC", "-DFMT_HEADER_ONLY", "-DSANKHYA_ENABLE_CUDA",
             "-DSANKHYA_MIN_COMPUTE_ARCH=103", f"-I{ref}/include", f"-I{ref}/src",
             f"-I{ROOT}/include", f"-I{ROOT}/oracle/ref/standin", "-isystem", torch_inc]
    seam = os.path.join(ROOT, "sih-26_gb300", "seam")
    sources = [os.path.join(seam, f + ".cpp")
               for f in ("pdhg_gpu", "pdhg_multi_gpu", "gpu_memory", "device")]
    sources += [os.path.join(ROOT, "tests", "host", f)
                for f in ("seam_standin.cpp", "checkpoint_stub.cpp")]
    core = os.path.join(ROOT, "oracle", "_ref", "libsankhya_core.a")
    return flags, sources, core


@pytest.fixture(scope="session")
def reference_core_library(tmp_path_factory):
    """libsankhya.so built from the reference's core with the seam in place of src/gpu and
    the CPU stand-in behind the engine's C ABI: what the reference's own Python package
    (bindings/python/sankhya) loads through SANKHYA_LIBRARY."""
    import subprocess

    flags, sources, core = core_link_args()
    lib = str(tmp_path_factory.mktemp("reference_core") / "libsankhya.so")
    cmd = (["g++", "-shared"] + flags + sources +
           ["-Wl,--whole-archive", core, "-Wl,--no-whole-archive", "-Wl,--no-undefined",
            "-fopenmp", "-lz", "-o", lib])
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-2000:]
    return lib
