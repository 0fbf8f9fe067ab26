"""The N > 1 path of bench.py on CPU: world_size-2 gloo ranks (replicas only -- planes x
scenarios shard with no data-path collective; the collectives are the max over ranks of the
timed region and the sum of the ranks' plane-seconds, after it).  No GPU is used."""
import json
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


def _worker(rank, world, port, q):
    import importlib.util

    import numpy as np
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    sys.path.insert(0, os.path.join(ROOT, "planes-rl_gb300"))
    import pe

    class A:
        seed, pop = 2, 64

    g = pe.random_genomes(bench.rank_genome_seed(A, rank), A.pop)
    t = bench.max_over_ranks(1.0 + rank, dist)  # rank r "took" 1 + r seconds
    u = bench.sum_over_ranks(100.0 + rank, dist)  # and flew 100 + r plane-seconds per step
    v = bench.job_value(u, 3, t)
    q.put((rank, g, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_take_the_slowest_time(built_lib):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (_, g0, t0, v0), (_, g1, t1, v1) = res
    # each rank flies its own population (weak scaling): no genome is shared
    assert not (g0[:, None, :] == g1[None, :, :]).all(axis=2).any()
    assert t0 == t1 == 2.0  # the slowest rank's time
    assert v0 == v1 == (100.0 + 101.0) * 3 / 2.0  # every rank's units over that time


def test_reference_arm_under_torchrun_prints_one_line(built_lib):
    """bench.py --impl reference with two ranks: rank 0 alone runs the CPU arm and prints one
    JSON line; rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--pop", "40", "--nseeds", "2",
           "--cpu-planes", "40", "--max-steps", "600"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_bench_host_top_k_matches_stable_sort():
    """bench.py's end-to-end generation picks the holdout's genomes on the host with an O(n)
    top-k; it must return what a stable descending sort returns (ties to the lower index)."""
    import importlib.util

    import numpy as np

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    rng = np.random.default_rng(0)
    for _ in range(300):
        n = int(rng.integers(1, 3000))
        s = rng.integers(0, 12, n).astype(np.float32)  # many ties
        s[rng.integers(0, n, n // 5)] = -100.0
        k = int(rng.integers(1, min(n, 16) + 1))
        np.testing.assert_array_equal(bench.top_k_host(s, k), np.argsort(-s, kind="stable")[:k])
