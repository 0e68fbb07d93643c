"""The multi-rank path of bench.py on CPU: two gloo ranks, replicas only.

Each rank runs its own system; the ranks exchange nothing on the data path,
only the barrier around the timed region and the max of their device times,
from which rank 0 reports the whole-job rate."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import io
    import contextlib
    import bench
    w, r, local = bench.dist_init()
    bench.barrier(w)
    ms = 10.0 * (r + 1)  # rank 1 is the slower one
    value, ms_max = bench.aggregate(w, 1000, 50, ms)
    # the reference arm: rank 0 alone runs; the others return without output
    out = io.StringIO()
    if r != 0:
        class A:
            steps, warmup = 1, 1
        with contextlib.redirect_stdout(out):
            bench.run_reference(A(), w, r)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, w, value, ms_max, out.getvalue()))


def test_two_gloo_ranks_aggregate_and_reference_arm():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, value, ms_max, out in res:
        assert w == 2 and ms_max == 20.0
        assert abs(value - 2 * 1000 * 50 / 0.020) < 1e-6
        if r == 1:
            assert out == ""
