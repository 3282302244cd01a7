"""The replica (multi-process) path of bench.py on CPU: two gloo ranks on
127.0.0.1 share a barrier and take the max of their times, and under the
reference arm only rank 0 works and prints."""
import importlib.util
import multiprocessing as mp
import os
import socket
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    try:
        b = _bench()
        d = b.Dist()
        d.barrier()
        m = d.max(float(rank + 1) * 1.5)
        d.barrier()
        d.close()
        q.put((rank, d.world, m))
    except Exception as e:  # reported to the parent
        q.put((rank, -1, repr(e)))


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert out == [(0, 2, 3.0), (1, 2, 3.0)], out


def test_single_process_needs_no_process_group():
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    b = _bench()
    d = b.Dist()
    assert d.world == 1 and d.rank == 0
    d.barrier()
    assert d.max(2.5) == 2.5
    d.close()
