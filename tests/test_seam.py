"""The drop-in C++ seam (sih-26_gb300/seam/) inside SANKHYA's tree: each file is checked
against the reference's own headers (src/gpu/*.hpp, include/sankhya/*.hpp), which is how a
maintainer builds it in place of src/gpu/*.cu, and the seam's behaviour is checked against
the reference's own solve_pdhg (see the last test). Needs the reference tree and g++."""
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


def test_seam_solves_like_the_reference(tmp_path):
    """`tests/host/seam_check.cpp`: the seam linked with the reference's own compiled sources
    and a CPU stand-in for the engine's C ABI that runs the reference PDHG. Its Solution must
    equal the reference's solve_pdhg bit for bit, and the model-error, no-engine, interrupt
    and logging paths must behave as the seam's contract says."""
    if not os.path.isdir(os.path.join(REF, "src", "gpu")) or shutil.which("g++") is None:
        pytest.skip("the reference tree (or g++) is not present here")
    import torch

    pyoracle.build(reference=True)
    objs = []
    for dirpath, _, files in os.walk(os.path.join(ROOT, "oracle", "_ref", "obj", "src")):
        objs += [os.path.join(dirpath, f) for f in files if f.endswith(".o")]
    assert objs, "the reference objects were not built"
    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    exe = str(tmp_path / "seam_check")
    cmd = (["g++", "-std=c++20", "-O1", "-DFMT_HEADER_ONLY", "-DSANKHYA_MIN_COMPUTE_ARCH=103",
            f"-I{REF}/include", f"-I{REF}/src", f"-I{ROOT}/include",
            f"-I{ROOT}/oracle/ref/standin", "-isystem", torch_inc,
            os.path.join(SEAM, "pdhg_gpu.cpp"),
            os.path.join(ROOT, "tests", "host", "seam_standin.cpp"),
            os.path.join(ROOT, "tests", "host", "seam_check.cpp")] + sorted(objs) +
           ["-fopenmp", "-o", exe])
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-2000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-2000:]
    assert run.stdout.strip().endswith("OK"), run.stdout
