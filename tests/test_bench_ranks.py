"""The benchmark's multi-GPU replica logic on CPU: two gloo ranks (127.0.0.1) reduce their timings to the slowest
rank's, the whole-job rate counts every replica's work, and under torchrun the reference arm runs on rank 0 only."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    times = [1.0 + rank, 5.0 - rank]                  # rank 0: (1, 5), rank 1: (2, 4)
    bench._sync_ranks(2, device="cpu")
    mx = bench._max_over_ranks(times, 2, device="cpu")
    bench._sync_ranks(2, device="cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"max": mx, "rate": bench._aggregate_rate(2, 1000, 3, mx[0])}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time(tmp_path):
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    assert res[0]["max"] == res[1]["max"] == [2.0, 5.0]
    assert res[0]["rate"] == pytest.approx(2 * 1000 * 3 / 2.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_never_loads_the_library():
    """The reference arm runs the oracle on its own set-up: neither the package nor libdpg_gb300.so is loaded."""
    code = (
        "import sys, json, argparse; sys.path.insert(0, %r)\n"
        "import bench\n"
        "bench.WORKLOAD['n_elem'] = (4, 4, 2)\n"
        "bench.run_reference(argparse.Namespace(steps=2, warmup=3))\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'dpgsolver_gb300' not in sys.modules, 'package imported'\n"
        "assert 'libdpg_gb300' not in maps, 'library mapped'\n"
        "assert 'liboracle_dg' in maps\n" % ROOT)
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
