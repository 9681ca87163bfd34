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


def test_tile_and_window_layouts(tmp_path):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is not available")
    sys.path.insert(0, os.path.join(ROOT, "sih-26_gb300"))
    from sankhya_gb300 import _paths, build

    build.build_engine()
    objdir = os.path.join(os.path.dirname(_paths.ENGINE_LIB), "obj")
    objs = [os.path.join(objdir, s.replace(".cu", ".o")) for s in build.CUDA_SOURCES]
    exe = str(tmp_path / "layout_check")
    cmd = ([nvcc] + build.ARCH +
           ["-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", _paths.INCLUDE_DIR, "-I",
            _paths.CSRC_DIR, os.path.join(ROOT, "tests", "host", "layout_check.cu")] + objs +
           ["-lcudart", "-o", exe])
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout
    run = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout
    assert run.stdout.startswith("OK"), run.stdout
