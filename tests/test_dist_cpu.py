"""CPU, two processes over gloo: the bench's multi-rank logic -- the job time
is the slowest rank's, the value counts every rank's numbers (weak scaling),
and the reference arm prints from rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_rank = 2.0 + rank  # rank 1 is the slower one
    ms, value = bench.aggregate(ms_rank, 1000, world)
    out[rank] = (ms, value, bench.barrier_max(float(rank), world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    for rank in range(world):
        ms, value, mx = res[rank]
        assert ms == 3.0 and mx == 1.0
        assert value == pytest.approx(2 * 1000 / 3e-3 / 1e6)


def _ref_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import contextlib
    import io
    import types

    import bench
    buf = io.StringIO()
    calls = []
    bench.cpu_baseline = lambda threads=None, scale=1.0, every_op=True: (calls.append(scale) or (1.0, 1, "stub", {}))
    bench.cpu_ops = lambda threads=None, scale=1.0, which=None: ({}, 1)
    with contextlib.redirect_stdout(buf):
        bench.run_reference(types.SimpleNamespace(gpus=world, steps=2, warmup=1))
    out[rank] = (buf.getvalue(), len(calls))


def test_reference_arm_runs_on_rank_zero_only():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_ref_worker, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert '"impl": "reference"' in res[0][0] and res[0][1] == 3
    assert res[1] == ("", 0)
