"""The allocation-free device product (sankhya_gb300_pdhg_spmv_noalloc) against the host
product (sankhya_gb300_pdhg_spmv): the same kernel over the same tiles and grid, so the
results must agree bit for bit, on two calls in a row (the second reuses the fixed scratch
and its counter, which the first must have put back to zero). The file is collected last, so
it runs after every other GPU test; it also passes alone in a fresh process, where its first
call does the scratch setup.
"""
import numpy as np
import pytest

from sankhya_gb300 import capi
from sankhya_gb300.model import LP


def _lp_with_long_row(m=60, n=6000, seed=4):
    """Row 0 touches every column (6000 entries: three chunks of a 2048-entry tile), so the
    products go through the chunk partials and the completion counter; the other rows are
    short."""
    rng = np.random.default_rng(seed)
    starts, rows, vals = [0], [], []
    for _ in range(n):
        r = sorted({0} | set(rng.integers(1, m, size=3).tolist()))
        rows += r
        vals += rng.normal(size=len(r)).tolist()
        starts.append(len(rows))
    return LP(m, n, np.array(starts, np.int32), np.array(rows, np.int32), np.array(vals),
              rng.normal(size=n), np.zeros(n), np.full(n, 10.0), np.full(m, -1.0),
              np.full(m, 1.0))


@pytest.mark.gpu
@pytest.mark.parametrize("scaled", [False, True])
def test_noalloc_matches_host_product_twice(scaled):
    torch = pytest.importorskip("torch")
    lp = _lp_with_long_row()
    rng = np.random.default_rng(5)
    with capi.PdhgEngine(0) as eng:
        eng.load(lp)
        if scaled:
            eng.scaling(0)
        stream = torch.cuda.Stream()
        for call in range(2):
            for op, n_in, n_out in ((0, lp.cols, lp.rows), (1, lp.rows, lp.cols)):
                v = rng.standard_normal(n_in)
                want = eng.spmv(op, v, scaled=scaled)
                dv = torch.from_numpy(v).to("cuda")
                out = torch.full((n_out,), float("nan"), dtype=torch.float64, device="cuda")
                torch.cuda.synchronize()
                eng.spmv_device(op, dv.data_ptr(), out.data_ptr(), scaled=scaled,
                                stream=stream.cuda_stream)
                stream.synchronize()
                got = out.cpu().numpy()
                assert np.array_equal(got, want), (call, op, float(np.abs(got - want).max()))


@pytest.mark.gpu
def test_noalloc_refuses_bad_arguments():
    lp = _lp_with_long_row(m=20, n=100)
    with capi.PdhgEngine(0) as eng:
        eng.load(lp)
        with pytest.raises(capi.EngineError):
            eng.spmv_device(2, 16, 16)  # no such product
        with pytest.raises(capi.EngineError):
            eng.spmv_device(0, 0, 0)  # null device buffers
        with pytest.raises(capi.EngineError):
            eng.spmv_device(0, 16, 16, scaled=True)  # nothing scaled yet
