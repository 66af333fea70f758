"""bench.py's multi-GPU aggregation (replicas of the workload, one per rank) on CPU: two gloo ranks
report different times; every rank sees the slowest, and the whole-job rate counts both ranks'
units over it."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
  os.environ["MASTER_ADDR"] = "127.0.0.1"
  os.environ["MASTER_PORT"] = str(port)
  dist.init_process_group("gloo", rank=rank, world_size=world)
  try:
    import bench

    ms = bench.max_over_ranks(100.0 + 50.0 * rank)
    out[rank] = (ms, bench.aggregate_rate(1.0e6, ms, world))
  finally:
    dist.destroy_process_group()


def test_slowest_rank_and_whole_job_rate():
  ctx = mp.get_context("spawn")
  with ctx.Manager() as manager:
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
      p.start()
    for p in procs:
      p.join(timeout=120)
      assert p.exitcode == 0
    for r in range(2):
      ms, rate = out[r]
      assert ms == 150.0
      assert rate == pytest.approx(2 * 1.0e6 / 0.150 / 1e6)


def test_single_process_is_the_identity():
  import bench

  assert bench.max_over_ranks(12.5) == 12.5
  assert bench.aggregate_rate(3.0e6, 1000.0, 1) == pytest.approx(3.0)
