"""Host-side layout invariants the kernels' shared-memory bounds rely on.

`tests/host/layout_check.cu` is built against the engine's own objects (the same
`build_tiles`, `build_windows`, `wide_lanes` and `graph_kernel_launches` the engine uses) and
run on the CPU. It checks tile coverage and limits, that every bulk copy fits its buffer and
its padded source, window alignment and capacity, and the staged-entry count, on random and
banded patterns with empty rows and rows at, just over and far over the tile capacity. The
engine builds tiles with exactly these calls in `Engine::load` (`csrc/engine.cu`).
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is not available")
    sys.path.insert(0, os.path.join(ROOT, "sih-26_gb300"))
    from sankhya_gb300 import _paths, build

    build.build_engine()
    objdir = os.path.join(os.path.dirname(_paths.ENGINE_LIB), "obj")
    objs = [os.path.join(objdir, s.replace(".cu", ".o")) for s in build.CUDA_SOURCES]
    exe = str(tmp_path_factory.mktemp("layout") / "layout_check")
    cmd = ([nvcc] + build.ARCH +
           ["-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", _paths.INCLUDE_DIR, "-I",
            _paths.CSRC_DIR, os.path.join(ROOT, "tests", "host", "layout_check.cu")] + objs +
           ["-lcudart", "-o", exe])
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout
    return exe


def _run(args):
    run = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout
    assert run.stdout.startswith("OK"), run.stdout
    return run.stdout


def test_tile_and_window_layouts(checker):
    _run([checker])


def _dump(path, ptr, idx, lines, extent):
    import numpy as np

    with open(path, "wb") as f:
        np.array([lines, extent], dtype=np.int32).tofile(f)
        np.asarray(ptr, dtype=np.int32).tofile(f)
        np.asarray(idx, dtype=np.int32).tofile(f)


def test_zipf_layouts(checker, tmp_path):
    """The engine's layouts (FP64 and FP32, at the window capacities) for the load-balance
    stress pattern: Zipf(1.5) row lengths, rows of thousands of entries cut into chunk
    tiles. A tenth of the 500,000 x 1,000,000, 3e7-nonzero case by default; the full size
    with SANKHYA_GB300_FULL_ZIPF=1 (about 1 GB of host memory)."""
    sp = pytest.importorskip("scipy.sparse")
    from sankhya_gb300 import build, lpgen

    build.build_lpgen()
    scale = 1 if os.environ.get("SANKHYA_GB300_FULL_ZIPF") == "1" else 10
    lp = lpgen.planted_zipf(500000 // scale, 1000000 // scale, 30000000 // scale, seed=3)
    csr = sp.csc_matrix((lp.values, lp.row_index, lp.col_starts),
                        shape=(lp.rows, lp.cols)).tocsr()
    csr.sort_indices()
    rows, cols = str(tmp_path / "rows.bin"), str(tmp_path / "cols.bin")
    _dump(rows, csr.indptr, csr.indices, lp.rows, lp.cols)
    _dump(cols, lp.col_starts, lp.row_index, lp.cols, lp.rows)
    out = _run([checker, rows])
    assert "chunk tiles" in out and not out.split(",")[-1].strip().startswith("0 ")
    _run([checker, cols])


def test_model_checks_follow_the_reference(tmp_path):
    """`tests/host/validate_check.cu`: the engine's model checks (validate_lp, run by both
    load entry points) accept a valid LP with infinite bounds, empty lines and explicit zeros,
    and refuse, with the model-error code, every numeric defect the reference's
    Model::validate refuses (src/core/model.cpp:127-240), the CSC defects a frozen matrix
    cannot hold, and an infinite cost (the engine's own rule)."""
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is not available")
    sys.path.insert(0, os.path.join(ROOT, "sih-26_gb300"))
    from sankhya_gb300 import _paths, build

    build.build_engine()
    objdir = os.path.join(os.path.dirname(_paths.ENGINE_LIB), "obj")
    objs = [os.path.join(objdir, s.replace(".cu", ".o")) for s in build.CUDA_SOURCES]
    exe = str(tmp_path / "validate_check")
    cmd = ([nvcc] + build.ARCH +
           ["-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", _paths.INCLUDE_DIR, "-I",
            _paths.CSRC_DIR, os.path.join(ROOT, "tests", "host", "validate_check.cu")] + objs +
           ["-lcudart", "-o", exe])
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout
    _run([exe])
