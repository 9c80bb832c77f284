"""Host logic of bench.py at more than one rank, on the CPU over gloo.

Cloths are independent, so N GPUs run N replicas of the workload with no
exchange on the data path; the ranks only meet at barriers and take the
largest time.  Both are checked here with two gloo ranks, and so is the
reference arm under torchrun, where rank 0 alone runs and prints."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, values, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        bench.barrier(2)
        out.put((rank, bench.max_over_ranks(values[rank], 2)))
        bench.barrier(2)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    values = [12.5, 40.25]
    procs = [ctx.Process(target=_rank_main, args=(r, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 40.25, 1: 40.25}


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    bench.barrier(1)
    assert bench.max_over_ranks(3.0, 1) == 3.0


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--steps", "1", "--warmup", "0", "--cloths", "3", "--ref-cloths", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["value"] == line["value"]
