"""The C-ABI library: it loads without a GPU and exports every symbol include/sankhya_gb300.h
declares; pure-arithmetic entry points answer on the CPU; device calls fail loudly (no
fallback) where no GPU is present."""
import ctypes
import os
import re

import pytest

from sankhya_gb300 import _paths, capi


def _declared_symbols():
    text = open(os.path.join(_paths.INCLUDE_DIR, "sankhya_gb300.h")).read()
    return sorted(set(re.findall(r"SGB_API\s+[\w\s\*]+?\b(sankhya_gb300_\w+)\s*\(", text)))


def test_header_declares_the_planned_entry_points():
    names = _declared_symbols()
    assert "sankhya_gb300_pdhg_solve" in names
    assert len(names) >= 12


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(capi.library_path())
    missing = [n for n in _declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(capi.EXPORTS) == sorted(_declared_symbols())


def test_memory_estimate_is_arithmetic(built):
    small = capi.estimate_memory(10, 20, 50)
    big = capi.estimate_memory(1_000_000, 2_000_000, 20_000_000)
    assert small < big
    # 4 value copies + 2 index copies per nonzero dominate at scale.
    assert big > 20_000_000 * (4 * 8 + 2 * 4)
    assert capi.estimate_memory(1000, 2000, 10000, "mixed") > capi.estimate_memory(1000, 2000, 10000)
    assert capi.estimate_memory(-1, -1, -1) > 0


def test_no_gpu_means_an_error_not_a_fallback(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.EngineError) as err:
        capi.PdhgEngine(0)
    assert err.value.code == 7
