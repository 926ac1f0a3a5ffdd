"""The multi-GPU path of bench.py is replicas only (one independent system
per rank, no data-path collective): a gloo barrier around the timed region and
max-over-ranks timing.  Checked here on CPU with world_size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    import bench
    r, w = bench.dist_setup()
    bench.barrier(w)
    slowest = bench.allreduce_max(1.0 + rank, w)   # per-rank timings -> the job's time
    args = type("A", (), {"n_lipid": 1000, "steps": 1, "warmup": 0, "gpus": w})()
    rc = bench.run_reference(args, r, w) if r != 0 else 0   # non-zero ranks print nothing, exit 0
    bench.barrier(w)
    out.put((r, w, slowest, rc))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_take_the_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert all(p.exitcode == 0 for p in procs)
    assert [r[:2] for r in res] == [(0, 2), (1, 2)]
    assert all(r[2] == 2.0 for r in res)      # max over ranks
    assert all(r[3] == 0 for r in res)
