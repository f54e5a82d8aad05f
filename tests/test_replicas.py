"""Host logic of the multi-GPU form ("replicas only"): two gloo ranks on CPU
run the bench's barrier and whole-job throughput aggregation."""
import importlib.util
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    import torch
    import torch.distributed as dist
    w, r, _ = bench.dist_init()
    bench.barrier(w)
    # rank r processed (r+1) million particle-steps in (1 + r) seconds
    v = bench.replica_throughput((r + 1) * 1e6, 1.0 + r, w, torch.device("cpu"))
    q.put((r, w, v))
    dist.destroy_process_group()


def test_two_replicas_sum_units_over_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
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
    assert [o[1] for o in out] == [2, 2]
    for _, _, v in out:
        assert v == pytest.approx(3e6 / 2.0)
