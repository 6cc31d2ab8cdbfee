"""The bench's multi-rank logic on CPU: two gloo ranks (127.0.0.1), each with
its own particles (weak scaling, no data-path collective); the timing is the
maximum over ranks and the reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    r, w, d = bench.dist_setup(None)
    assert (r, w) == (rank, ws) and d is not None
    t_dev, t_e2e = bench.max_over_ranks(d, 1.0 + rank, 5.0 - rank)   # each rank its own times
    # the reference arm: ranks other than 0 return at once without work
    ref = bench.run_reference(None, r, w, d) if r != 0 else None
    out.put((rank, t_dev, t_e2e, ref, bench.units_total(1000, w)))
    d.barrier()
    d.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_sum_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, t_dev, t_e2e, ref, units in res:
        assert t_dev == 2.0 and t_e2e == 5.0          # max over ranks, on every rank
        assert ref is None
        assert units == 2000                           # whole-job units: the ranks' batches add up


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(None, 3.0, 4.0) == (3.0, 4.0)
    assert bench.units_total(7, 1) == 7
