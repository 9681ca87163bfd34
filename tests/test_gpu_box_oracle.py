"""The oracle against the reference's own PDHG on the GPU machine's own CPU architecture.

The CPU tests (tests/test_oracle_vs_reference.py) pin the oracle bit for bit to the
reference's build where the reference tree is, on x86-64. The GPU machine is aarch64 and has
no reference tree: there the reference library is built from the staged copy of its sources
(`make -C oracle stage` / `pyoracle.build`), and these tests repeat the bit-for-bit checks,
so the oracle that checks the engine and the CPU baseline that the bench times are pinned on
that architecture too. They need no GPU; they are marked `gpu` because they run where the GPU
tests run. On x86-64 they skip (the CPU tests cover it).
"""
import platform

import pytest

import test_oracle_vs_reference as pinned

pytestmark = pytest.mark.gpu


def _off_x86():
    if platform.machine() in ("x86_64", "AMD64"):
        pytest.skip("pinned on x86-64 by tests/test_oracle_vs_reference.py")


@pytest.mark.parametrize("name,lp,kw", list(pinned._cases()), ids=[c[0] for c in pinned._cases()])
def test_solve_is_bit_identical_here(reference, oracle, name, lp, kw):
    _off_x86()
    pinned.test_solve_is_bit_identical(reference, oracle, name, lp, kw)


@pytest.mark.parametrize("make", [c[1] for c in pinned._SCALING_CASES],
                         ids=[c[0] for c in pinned._SCALING_CASES])
def test_scaling_and_evaluate_are_bit_identical_here(reference, oracle, make):
    _off_x86()
    pinned.test_scaling_and_norm_are_bit_identical(reference, oracle, make)
    pinned.test_evaluate_is_bit_identical(reference, oracle, make)
