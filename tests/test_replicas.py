"""bench.py's multi-GPU path is replicas only: one process per GPU, its own
scenes, the process group only for the barrier and the max/sum reductions of
the timing.  Two gloo ranks on the CPU run that logic."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    D = bench.Dist()
    D.barrier()
    # rank r: 1000*(r+1) particles, (10 + r) ms for 5 steps
    value, ms_max = bench.aggregate(D, 1000 * (rank + 1), 5, 10.0 + rank)
    D.close()
    q.put((rank, value, ms_max))


def test_two_replicas_gloo():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    # whole job: (1000 + 2000) particles * 5 steps / max(10, 11) ms
    for _, value, ms_max in out:
        assert ms_max == 11.0
        assert abs(value - 3000 * 5 / 0.011) < 1e-6
