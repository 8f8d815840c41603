"""The bench's replica path for N > 1, on the CPU: two gloo ranks agree on the max-over-ranks
clock and on the whole-job value; a rank that leaves before the collective is detected by
the other rank through a short process-group timeout (no GPU involved)."""
import os
import socket
import sys
from datetime import timedelta
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, times, leave, out):
    sys.path.insert(0, str(ROOT))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as td

    import bench

    td.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=5))
    if rank == leave:  # this rank leaves between steps, before the timing collective
        out.put((rank, "left", None))
        return
    try:
        ms = bench.replica_max(td, times[rank])
        out.put((rank, ms, bench.replica_value(world, 5, 50, ms)))
        td.barrier()
        td.destroy_process_group()
    except RuntimeError as exc:
        out.put((rank, "error", str(exc)[:200]))


def _run(times, leave=-1):
    import torch.multiprocessing as mp

    world = len(times)
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, times, leave, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(60)
        if p.is_alive():
            p.kill()
    return res, [p.exitcode for p in procs]


@pytest.mark.timeout(300)
def test_replica_clock_is_the_max_over_ranks():
    res, codes = _run([12.5, 20.0])
    assert codes == [0, 0]
    for rank, ms, value in res:
        assert ms == 20.0
        assert value == pytest.approx(2 * 5 * 50 / 0.020)


@pytest.mark.timeout(300)
def test_a_rank_that_leaves_is_detected_by_the_timeout():
    res, _ = _run([12.5, 20.0], leave=1)
    by_rank = dict((r, (a, b)) for r, a, b in res)
    assert by_rank[1][0] == "left"
    assert by_rank[0][0] == "error"  # the collective ended with an error instead of hanging
