"""The multi-GPU path of bench.py is replicas only (no collective on the data
path): each rank serves its own seeded requests and the whole-job figures
are all ranks' work over the slowest rank's time.  These tests run that
aggregation with world_size 2 on the CPU (gloo, 127.0.0.1).  No GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_rank = [0.25, 0.75][rank]                  # this rank's time (s)
        t = bench.rank_max(t_rank, dist, "cpu")
        rate = bench.whole_job_rate(1000, world, t)
        cases = bench.batch_cases(2, seed=bench.rank_seed(rank))
        alfas = [float(c[1].alfa) for c in cases]
        out.put((rank, t, rate, alfas))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_gloo_world2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, t0, rate0, a0), (r1, t1, rate1, a1) = res
    assert t0 == t1 == 0.75                 # both ranks see the slowest rank's time
    assert rate0 == rate1 == 2 * 1000 / 0.75   # all ranks' units over that time
    assert a0[1] != a1[1]                   # each rank serves its own seeded requests


def test_bench_gpus2_spawns_two_replicas_gloo():
    """`bench.py --gpus 2` outside a launcher starts two replica processes
    itself (torch.distributed.run, 127.0.0.1); in the CPU check mode each
    rank times its own seeded request over gloo and rank 0 prints the
    whole-job line."""
    import json
    import subprocess
    pytest.importorskip("torch")
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR",
                                                            "MASTER_PORT")}
    env["OMP_NUM_THREADS"] = "1"
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--batch", "2",
                        "--cpu-replica-check"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2
    assert line["value"] == pytest.approx(2 * line["units_per_rank"] / line["seconds"])
    a0, a1 = line["alfas"]
    assert len(a0) == len(a1) == 2 and a0[1] != a1[1]     # each rank its own seeded requests


def test_bench_reference_arm_line():
    """`bench.py --impl reference` (the oracle on the host cores, no GPU and
    no product library) prints one JSON line with the contract's keys: the
    same metric, unit and config as the GPU arm, a cpu_baseline describing
    the run and an e2e without copies."""
    import json
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--batch", "2", "--ref-seconds", "1"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["unit"] == "cell-updates/s" and line["dtype"] == "f64" and line["n_gpus"] == 1
    assert "513x129" in line["config"]["workload"] and line["config"]["batch_per_gpu"] == 2
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["sample"]
    assert cpu["value"] == line["value"]
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
