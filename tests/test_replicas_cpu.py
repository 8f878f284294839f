"""The multi-GPU path of bench.py on CPU: N independent replicas (no
data-path collective), a barrier around the timed region and the maximum of
the ranks' times, here over world_size 2 gloo ranks; and the reference arm
under the launcher, where rank 0 alone runs and prints."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.dist_init()
    bench.barrier(w)
    slowest = bench.reduce_max(10.0 + 5.0 * r, w)  # rank 1 is the slower one
    q.put((r, w, local, slowest, bench.replica_value(w, 1000, 4, slowest)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_barrier_and_slowest_time():
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
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)  # both ranks see the slowest time
    assert all(abs(o[4] - 2 * 1000 * 4 / 15e-3) < 1e-6 for o in out)


@pytest.mark.skipif(not (ROOT / "oracle" / "_build" / "libbhoracle.so").exists(), reason="oracle not built")
def test_reference_arm_under_launcher_rank0_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--bodies", "3000", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["e2e"]["h2d_bytes_per_step"] == 0
