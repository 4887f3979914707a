"""bench.py's replica logic (N independent brains, one per rank) with gloo ranks on CPU:
barrier + max-over-ranks timing, and the reference arm running on rank 0 only."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), AXC_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(world)
    d.barrier()
    t = d.max(1.0 + rank)                 # per-rank elapsed times 1.0 and 2.0
    q.put((rank, d.world, d.rank, t))
    d.close()


def test_two_gloo_ranks_take_the_max():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2, 2]
    assert [r[3] for r in res] == [2.0, 2.0]


def _ref_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), AXC_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import io
    import contextlib
    import bench
    sys.argv = ["bench.py", "--impl", "reference", "--workload", "plain-16k", "--steps", "2", "--warmup", "1",
                "--gpus", str(world)]
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.main()
    q.put((rank, buf.getvalue()))


def test_reference_arm_prints_on_rank0_only():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_ref_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(300)
        assert p.exitcode == 0
    out = dict(q.get(timeout=10) for _ in range(2))
    assert '"impl": "reference"' in out[0]
    assert out[1].strip() == ""
