"""The multi-process side of bench.py, on CPU with gloo: replicas only, so the
only cross-rank step is the max-over-ranks of the timed region, and the
reference arm runs on rank 0 alone."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total = bench.max_over_ranks(torch, tdist, 10.0 * (rank + 1), "cpu")
        out[rank] = (total, bench.job_gkeys_per_s(1 << 28, 20, world, total))
    finally:
        tdist.destroy_process_group()


def test_max_over_ranks_world_2():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    # both ranks see the slower rank's time and the same whole-job rate
    assert res[0] == res[1]
    total, rate = res[0]
    assert total == 20.0
    assert rate == pytest.approx(2 * (1 << 28) * 20 / 0.020 / 1e9)


def test_single_rank_needs_no_collective():
    assert bench.max_over_ranks(torch, None, 7.5, "cpu") == 7.5


def test_reference_arm_only_on_rank_0(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 1, 1, 2

    assert bench.run_reference(A()) is None
    assert capsys.readouterr().out == ""
