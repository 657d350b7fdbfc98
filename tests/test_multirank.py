"""World-size-2 CPU (gloo) tests of the benchmark's N > 1 path: replicas only,
a barrier around the timed region and the maximum time over ranks; under
torchrun the reference arm prints one line from rank 0 and the other rank
exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_available():
    try:
        import torch

        return torch.cuda.is_available()
    except ImportError:
        return False


# CPU-only: with a GPU the helpers pick NCCL and one device per rank
pytestmark = pytest.mark.skipif(_cuda_available(), reason="gloo tests of the multi-rank path run on CPU hosts")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, ws, _ = bench.dist_init()
    bench.barrier(ws)
    m = bench.max_over_ranks(1.5 + r, ws)
    out.put((r, ws, m, dist.get_backend()))
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_with_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r for r, *_ in res] == [0, 1]
    assert all(ws == 2 and m == 2.5 and be == "gloo" for _, ws, m, be in res)


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--gpus", "2",
           "--impl", "reference", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
