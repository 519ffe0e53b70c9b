"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1) take the slowest rank's times
and report the replicas' aggregate throughput, as the GPU run does over nccl."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as tdist
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    r, w = bench.env_rank()
    times = [10.0 * (rank + 1), 5.0 + rank]  # ms: device step, end-to-end step
    ms_max, e2e_max = bench.max_over_ranks(times, True, "cpu")
    tdist.barrier()
    q.put((r, w, ms_max, e2e_max, bench.replica_throughput(w, ms_max)))
    tdist.destroy_process_group()


def test_two_ranks_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    for _, _, ms_max, e2e_max, value in out:
        assert ms_max == 20.0 and e2e_max == 6.0
        assert value == pytest.approx(2 * 1000.0 / 20.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 4.0], False, "cpu") == [3.0, 4.0]
    assert bench.replica_throughput(1, 13.2) == pytest.approx(1000.0 / 13.2)
