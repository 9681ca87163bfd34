"""`bench.py --gpus 2` as two replicas over gloo, on the CPU.

The path does not shard: N ranks solve N independent copies of the LP, and the only
collectives are a barrier on each side of the timed region and a max of the step times. Two
ranks run `bench.main()` with stand-in device engines whose solve time depends on the rank.
Rank 0 must print the single line, with n_gpus = 2, the slower rank's time as `value` and the
whole-job LPs/s computed from it. Rank 1 must print nothing.
"""
import json
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytest.importorskip("torch.distributed")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    for sub in ("", "sih-26_gb300", "oracle", "tests"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": "0", "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    from sankhya_gb300 import capi
    import test_bench_contract as contract

    class RankEngine(contract.StandInPdhgEngine):
        def solve(self, precision="fp64", **kw):
            r = contract._Result(self.lp, precision)
            r.device_seconds = 0.09 + 0.02 * rank
            return r

    capi.PdhgEngine = RankEngine
    bench.WORKLOAD = dict(blocks=2, rows_per_block=300, cols_per_block=600, k=9, seed=2026)
    sys.argv = ["bench.py", "--gpus", str(world), "--steps", "1", "--warmup", "3",
                "--no-batch", "--no-adjoint", "--no-cpu-baseline", "--no-zipf", "--no-qp",
                "--no-reference-gpu"]
    with open(out_path, "w") as f:
        sys.stdout = f
        try:
            bench.main()
        finally:
            sys.stdout.flush()
            sys.stdout = sys.__stdout__


def test_two_replicas(tmp_path):
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    outs = [str(tmp_path / f"rank{r}.out") for r in range(world)]
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, outs[r])) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    lines0 = [l for l in open(outs[0]).read().splitlines() if l.startswith("{")]
    lines1 = [l for l in open(outs[1]).read().splitlines() if l.startswith("{")]
    assert len(lines0) == 1 and not lines1
    line = json.loads(lines0[0])
    assert line["n_gpus"] == 2
    assert line["value"] == pytest.approx(0.11)  # the slower rank's step
    assert line["lps_per_s"] == pytest.approx(2 / 0.11)
