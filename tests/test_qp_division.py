"""The QP row pass's division (Markstein's correction of the product with the correctly
rounded reciprocal, sih-26_gb300/csrc/qp_kernels.cu divide()) equals IEEE division bit for bit
on 20 million random pairs and hand-picked cases (tests/host/qp_division_check.c, run on the
CPU with C's correctly rounded fma)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_division_sequence_is_correctly_rounded(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    exe = str(tmp_path / "qp_division_check")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-std=c11", "-o", exe,
                    os.path.join(ROOT, "tests", "host", "qp_division_check.c"), "-lm"],
                   check=True)
    run = subprocess.run([exe, "20000000"], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout
    assert run.stdout.strip().startswith("0 of "), run.stdout
