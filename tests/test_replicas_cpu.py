"""bench.py's multi-process path on CPU ranks (gloo, world size 2): the
barrier / max-over-ranks helpers, and the reference arm under torchrun
printing exactly one JSON line, from rank 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup(world)
    bench.barrier(w)
    m = bench.max_over_ranks(w, float(rank + 1) * 0.5)
    with open(os.path.join(out, "rank%d.txt" % rank), "w") as f:
        f.write("%d %d %r" % (w, r, m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_dist_helpers_gloo_world2(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the CPU path runs where no GPU is visible")
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(2, free_port(), str(tmp_path)), nprocs=2,
                       start_method="spawn")
    for r in range(2):
        w, rr, m = open(os.path.join(tmp_path, "rank%d.txt" % r)).read().split()
        assert (int(w), int(rr), float(m)) == (2, r, 1.0)


def test_reference_arm_under_torchrun_prints_once(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the CPU path runs where no GPU is visible")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "1", "--ref-dims", "10"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # whole solves, measured: the 10^3 box converges to 1e-8 in tens of iterations
    assert 10 < line["iterations"]["min"] <= line["iterations"]["max"] < 200
    assert line["config"]["tol_rel"] == 1e-8 and line["config"]["nx"] == 10
