"""Host logic of bench.py on CPU: the multi-rank path (gloo, world size 2) and the roofline context.

Every rank of ``bench.py --gpus N`` is an independent replica of the whole
workload; ranks meet only at barriers and at the max-over-ranks reduction
of the timed region.  These tests run that reduction and the reference
arm's rank handling as real processes on the CPU."""
import importlib.util
import json
import os
import socket
import subprocess
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_multirank", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _bench()
        dist.barrier()
        seconds = [1.5, 2.5][rank]                     # rank 1 is the slow replica
        slowest = bench.max_over_ranks(seconds, world)
        rate = bench.job_rate(world, 1000, 5, slowest)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"slowest": slowest, "rate": rate}, f)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo_world_2(tmp_path):
    tmp.spawn(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for g in got:
        assert g["slowest"] == 2.5                     # every rank sees the slowest rank's time
        assert g["rate"] == 2 * 1000 * 5 / 2.5         # whole-job units over that time


def test_single_rank_needs_no_process_group():
    bench = _bench()
    assert not dist.is_initialized()
    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.job_rate(1, 10, 4, 2.0) == 20.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_bloch_roofline_counts_h_and_s_writes(tmp_path):
    bench = _bench()
    peaks = tmp_path / "peaks.json"
    peaks.write_text(json.dumps({"hbm_gbs": 8000.0}))
    r = bench.bloch_roofline(0.004, 10 ** 8, str(peaks))        # 2 * 16 bytes * 1e8 elements in 4 ms
    assert r["bytes_per_step"] == 32 * 10 ** 8 and r["achieved_gbs"] == 800.0 and r["frac"] == 0.1
    assert bench.bloch_roofline(0.0, 10 ** 8, str(peaks)) is None
    assert bench.bloch_roofline(0.004, 10 ** 8, str(tmp_path / "absent.json"))["frac"] is None


def test_ordinal_suffixes():
    bench = _bench()
    assert [bench.ordinal(n) for n in (1, 2, 3, 4, 11, 12, 13, 16, 21, 22, 23, 32, 101, 111)] == \
        ["1st", "2nd", "3rd", "4th", "11th", "12th", "13th", "16th", "21st", "22nd", "23rd", "32nd", "101st", "111th"]
