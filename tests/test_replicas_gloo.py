"""Multi-process path of bench.py on CPU (gloo, world size 2): the path
shards as independent replicas, so ranks share nothing but the barrier and
the max / sum reductions of the timing; every replica's result is the same."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    from oracle import Oracle

    from beam_gb300 import Graph
    d = bench.Dist()
    g = Graph.generate("dcsbm:n=1024,blocks=8,ratio=20,gamma=2.5,deg=20,seed=3")
    o = Oracle.from_graph(g, threads=1)
    o.run(20)
    merges = o.stats()["accepted_merges_after_validation"]
    d.barrier()
    mx = d.reduce(float(10 + rank), "max")
    total = d.reduce(float(merges), "sum")
    hashes = d.reduce(float(o.partition_hash() % 1000003), "max"), d.reduce(-float(o.partition_hash() % 1000003),
                                                                            "max")
    out.put((rank, mx, total, merges, hashes))
    d.close()


def test_two_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    results = [q.get(timeout=10) for _ in procs]
    for rank, mx, total, merges, (hmax, hneg) in results:
        assert mx == 11.0                       # slowest rank's time
        assert total == 2.0 * merges            # whole-job merges = sum over replicas
        assert hmax == -hneg                    # identical partitions on both replicas
