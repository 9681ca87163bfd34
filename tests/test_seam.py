"""The drop-in C++ seam (sih-26_gb300/seam/) compiles inside SANKHYA's tree: each file is
checked against the reference's own headers (src/gpu/*.hpp, include/sankhya/*.hpp), which is
how a maintainer builds it in place of src/gpu/*.cu. Needs the reference tree and g++."""
import os
import shutil
import subprocess

import pytest

import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEAM = os.path.join(ROOT, "sih-26_gb300", "seam")
REF = pyoracle.REFERENCE_TREE


@pytest.mark.parametrize("name", ["pdhg_gpu", "pdhg_multi_gpu", "gpu_memory", "device"])
def test_seam_compiles_against_reference_headers(name):
    if not os.path.isdir(os.path.join(REF, "src", "gpu")) or shutil.which("g++") is None:
        pytest.skip("the reference tree (or g++) is not present here")
    import torch

    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-DFMT_HEADER_ONLY",
           "-DSANKHYA_MIN_COMPUTE_ARCH=103", f"-I{REF}/include", f"-I{REF}/src",
           f"-I{ROOT}/include", f"-I{ROOT}/oracle/ref/standin", "-isystem", torch_inc,
           os.path.join(SEAM, name + ".cpp")]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-2000:]
