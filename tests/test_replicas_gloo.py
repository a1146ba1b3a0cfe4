"""The multi-GPU form of the benchmark is N independent replicas (the path
does not shard): each rank solves its own matrix, and the ranks only meet
at the timing barriers and the max-over-ranks of the step time.  That host
logic (bench.py's dist_env, barrier, allmax and the rank-0-only reference
arm) runs here as two gloo ranks on the CPU."""
import importlib.util
import os
import socket

import pytest

from tests.conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import io
    import contextlib

    import torch.distributed as dist

    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = b.dist_env()
    b.barrier(w)
    m = b.allmax(1.5 * (rank + 1), w)
    # the reference arm prints only on rank 0; other ranks return at once
    buf = io.StringIO()
    if rank != 0:
        with contextlib.redirect_stdout(buf):
            b.run_reference(type("A", (), {"nocc": 5, "nvirt": 19, "steps": 1, "warmup": 0})())
    b.barrier(w)
    dist.destroy_process_group()
    out.put((rank, r, w, local, m, buf.getvalue()))


def test_two_replicas_barrier_and_max():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, local, m, printed in res:
        assert (r, w, local) == (rank, 2, rank)
        assert m == 3.0              # the max over ranks, on every rank
        if rank == 1:
            assert printed == ""     # no line from the non-zero rank
