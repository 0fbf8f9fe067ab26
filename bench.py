#!/usr/bin/env python
"""Benchmark: simulated plane-seconds per second for one full generation at scale.

Workload (the configuration the headline metric is quoted on): 100,000 genomes drawn like the
reference's grand() from std::mt19937(2), each flown under 12 training scenarios (env seeds
2*12+s+1 = 25..36, vary 0, as the GA's generation 2 would), tail-aware score per genome, then
the top 8 genomes re-flown on a 128-scenario holdout (env seeds 3 + i*7919).  Up to 7200 steps
(12 s) per flight, the reference's horizon.  A "step" of this benchmark is that whole
generation.  Inputs are synthetic (no dataset exists for this path).

  value  plane-seconds/s with genomes resident in HBM (pe_eval_batch on device buffers)
  e2e    the same through pe_evaluate_population with pinned host buffers (copies included)
  ref_cuda the reference's own CUDA build on the same GPU and generation (its sim.cu compiled with its
         flags, driven as run_ga drives gpu_prepare / gpu_sim), host to host, with its own clock
         samples, its ratio to value / e2e and the parity of its distances and scores with this
         build's (a comparison leg like cpu_baseline, run after the timed region).
  grads  the second headline figure, grads/sec: d(objective)/d(genome) of 256 genomes (drawn from
         std::mt19937(4)) over 8 scenarios (env seeds 1..8), 3600 steps, a checkpoint every 60
         steps (pe_grad), against central finite differences (70 evaluations per genome) on the
         same GPU: FP64 (pe_objective, the precision the 1e-3 check needs), FP32 through the
         same smoothed model (pe_objective), and FP32 through the evaluation kernels (the fastest
         forward pass here) of the unsmoothed and of the smoothed distance; and the accuracy of
         pe_grad and of those FP32 differences against FP64 differences of every genome.
  hybrid the hybrid search: a 30-generation device GA at pop 16,384 x 8 scenarios whose top 64 genomes
         take 8 Adam steps (lr 1e-2, normalized units) on pe_grad every generation, against the same
         GA without them, for GA seeds 5..9; champions audited on 4,096 scenarios (9001 + i*7919);
         mean and sd over the seeds.
  configs the two smaller evaluation configurations as throughput figures (their parity is in the
         tests): 1,024 x 8 (genomes from std::mt19937(0), env seeds 1..8) and 8,192 x 8 (mt19937(1),
         seeds 9..16), 7200 steps, device-resident, each in the default shape (the whole flight in
         one launch), in 600-step (1 s) chunks replayed from a captured CUDA graph, and in the
         shape pe_autotune picks for the batch; then host to host, this build
         (pe_evaluate_population) beside the reference's own CUDA build on the same genomes and
         seeds (with its clock samples, the ratio and the parity of its distances and scores).

Plane-seconds = integrated 600 Hz steps of every flight / 600 (oversize meshes fly 0 steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "planes-rl_gb300")
ORACLE = os.path.join(ROOT, "oracle")
METRIC = "simulated plane-seconds/sec at pop 100k x 12"
UNIT = "plane-s/s"
# Algorithmic FP32 work of one plane-step (FMA = 2): the reference step's own count, 128 per
# panel (print warp, rotation of r and n, relative flow with rotation, normal force and skin
# friction, force and torque sums) plus ~300 per step (gusts, attitude matrix, integrator).
# roofline.achieved uses it.  The body-frame kernel needs less for the same physics: the
# print-warped normal is constant over a flight (staged once), so this formulation's own count
# is 103 per panel and 230 per step; roofline.formulation_count reports the fraction on it too.
FLOP_PER_PANEL_STEP = 128
FLOP_PER_STEP = 300
FLOP_PER_PANEL_STEP_BODY = 103
FLOP_PER_STEP_BODY = 230


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--pop", type=int, default=100000)
    ap.add_argument("--nseeds", type=int, default=12)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--holdout", type=int, default=128)
    ap.add_argument("--holdout-base", type=int, default=3)
    ap.add_argument("--topk", type=int, default=8)
    ap.add_argument("--max-steps", type=int, default=7200)
    ap.add_argument("--cpu-planes", type=int, default=2000, help="CPU baseline sample (genomes x all seeds)")
    ap.add_argument("--cpu-planes-1core", type=int, default=150, help="single-core CPU baseline sample")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-grads", action="store_true")
    ap.add_argument("--grad-pop", type=int, default=256)
    ap.add_argument("--grad-seeds", type=int, default=8)
    ap.add_argument("--grad-steps", type=int, default=3600)
    ap.add_argument("--grad-every", type=int, default=60, help="checkpoint interval")
    ap.add_argument("--fd64-genomes", type=int, default=64, help="FP64 finite-difference sample")
    ap.add_argument("--no-grad-accuracy", action="store_true", help="skip pe_grad vs FP64 differences")
    ap.add_argument("--no-hybrid", action="store_true")
    ap.add_argument("--hybrid-seeds", default="5,6,7,8,9", help="GA seeds of the hybrid-search comparison")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip the reference CUDA build's leg")
    ap.add_argument("--ref-cuda-reps", type=int, default=3, help="timed generations of the reference build")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def top_k_host(scores, k):
    """Indices of the k best scores, best first, ties to the lower index: the order of a stable
    descending sort, in O(n) (partition, then sort only the k)."""
    kth = scores[np.argpartition(-scores, k - 1)[k - 1]]
    above = np.flatnonzero(scores > kth)
    ties = np.flatnonzero(scores == kth)[:k - len(above)]
    top = np.concatenate([above, ties])
    return top[np.lexsort((top, -scores[top]))]


def rank_genome_seed(args, rank):
    """Weak scaling: every rank flies its own population of `pop` genomes, drawn from its own seed."""
    return args.seed + 1000003 * rank


def max_over_ranks(x, pg, device=None):
    """The job's time is the slowest rank's (no collective when pg is None)."""
    if pg is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, pg, device=None):
    """The units of the whole job: every rank flies its own population, so its count differs."""
    if pg is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def job_value(units_per_step_all_ranks, steps, seconds):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return units_per_step_all_ranks * steps / seconds


def training_seeds(args):
    return [args.seed * args.nseeds + s + 1 for s in range(args.nseeds)]


def holdout_seeds(args):
    return [args.holdout_base + i * 7919 for i in range(args.holdout)]


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(genomes, args, nthreads=None):
    """The oracle (OpenMP C restatement of the reference step) on a bounded sample."""
    sys.path.insert(0, ORACLE)
    import oracle_py

    n = min(args.cpu_planes, genomes.shape[0])
    nthreads = nthreads or os.cpu_count() or 1
    seeds = training_seeds(args)
    t0 = time.perf_counter()
    _, steps = oracle_py.eval_batch(genomes[:n], seeds, vary=0, max_steps=args.max_steps, nthreads=nthreads)
    el = time.perf_counter() - t0
    return {"value": float(steps.sum()) / 600.0 / el, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d genomes x %d scenarios (first genomes of the workload), %.1f s" % (n, len(seeds), el),
            "seconds": el}


def rank_avg(x):
    """Ranks with ties averaged (1-based), as Spearman's coefficient wants them."""
    x = np.asarray(x, np.float64)
    order = np.argsort(x, kind="mergesort")
    r = np.empty(len(x))
    r[order] = np.arange(1, len(x) + 1)
    _, inv, cnt = np.unique(x, return_inverse=True, return_counts=True)
    sums = np.bincount(inv, weights=r)
    return (sums / cnt)[inv]


def spearman(a, b):
    ra, rb = rank_avg(a), rank_avg(b)
    ra -= ra.mean()
    rb -= rb.mean()
    return float((ra * rb).sum() / np.sqrt((ra * ra).sum() * (rb * rb).sum()))


def ref_cuda_runner():
    """(runner executable, reference PTX, None), or (None, None, why not): the reference's sim.cu
    compiled to PTX where its sources are (oracle/_ref/ref_sim.ptx) and oracle/ref_cuda_runner,
    built here with g++ against libcuda."""
    ptx = os.path.join(ORACLE, "_ref", "ref_sim.ptx")
    if not os.path.exists(ptx):
        return None, None, ("oracle/_ref/ref_sim.ptx absent: the reference's sim.cu is compiled where its sources "
                            "are, and none was carried here")
    try:
        import importlib.util

        spec = importlib.util.spec_from_file_location("planes_oracle_build", os.path.join(ORACLE, "build.py"))
        obuild = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(obuild)
        return obuild.build_ref_cuda_runner(), ptx, None
    except Exception as e:  # the runner needs only g++ and libcuda
        return None, None, "oracle/ref_cuda_runner did not build: %s" % str(e).splitlines()[0]


def tail_scores(samples, nseeds):
    """The tail-aware score of src/sim.cu:340-357 (0.65 mean + 0.25 mean of the worst ceil(S/4) +
    0.10 worst) of plane-major samples, in float64: for ranking the reference build's planes."""
    x = np.sort(np.asarray(samples, np.float64).reshape(-1, nseeds), axis=1)
    k = (nseeds + 3) // 4
    return 0.65 * x.mean(axis=1) + 0.25 * x[:, :k].mean(axis=1) + 0.10 * x[:, 0]


def measure_ref_cuda(args, genomes, ours, device):
    """The reference's own CUDA build on this GPU, on the same generation (a comparison leg beside
    cpu_baseline, run after this build's timed region): the reference's src/sim.cu compiled with its
    flags to PTX (oracle/_ref/ref_sim.ptx, built where the reference sources are) and driven by
    oracle/ref_cuda_runner as run_ga drives gpu_prepare / gpu_sim (src/sim.cu:431-456): genomes H2D,
    prepare, per training seed 12 synced 600-step launches + D2H, tail-aware scores and top-k on the
    host, each of the top k flown on the holdout copies.  One warm-up generation, then `reps` timed
    host to host.  Parity of its distances and scores with this build's in the same line."""
    import tempfile

    exe, ptx, why = ref_cuda_runner()
    if why:
        return {"unavailable": why}
    pop, S, K, H = args.pop, args.nseeds, args.topk, args.holdout
    with tempfile.TemporaryDirectory() as tmp:
        gpath = os.path.join(tmp, "genomes.bin")
        np.ascontiguousarray(genomes, np.float32).tofile(gpath)
        clocks = Clocks(device)
        clocks.start()
        r = subprocess.run([exe, ptx, "gen", gpath, str(pop), "0", tmp, str(args.ref_cuda_reps), str(H),
                            str(args.holdout_base), str(K)] + [str(x) for x in training_seeds(args)],
                           capture_output=True, text=True)
        clk = clocks.stop()
        if r.returncode != 0:
            return {"unavailable": "reference runner failed (%d): %s" % (r.returncode, (r.stderr or r.stdout).strip()[-300:])}
        secs = [float(x) for x in open(os.path.join(tmp, "timing.txt")).read().split("seconds")[1].split()]
        ref = np.fromfile(os.path.join(tmp, "fitness.bin"), np.float32)
        ref_scores = np.fromfile(os.path.join(tmp, "scores.bin"), np.float32)
        ref_top = np.fromfile(os.path.join(tmp, "top.bin"), np.int32)
        ref_hold = np.fromfile(os.path.join(tmp, "holdout.bin"), np.float32).reshape(K, H)
    med = float(np.median(secs))
    value = ours["plane_s_per_gen"] / med
    d = ours["dist"]
    ok = ref > -100
    tol = 0.005 * np.maximum(np.abs(ref), 1.0)
    out = {
        "value": value, "unit": UNIT, "seconds_per_generation": secs, "reps": len(secs),
        "what": "the reference's k_prepare/k_sim (src/sim.cu, its flags -O3 -use_fast_math, PTX JIT-loaded) "
                "driven as run_ga drives gpu_prepare/gpu_sim: %d x %d generation + top-%d x %d holdout, host to "
                "host, same genomes and seeds; plane-seconds numerator from this build's step counts" % (pop, S, K, H),
        "ratio_e2e": ours["e2e_value"] / value,
        "ratio_device_resident": ours["value"] / value,
        "parity": {
            "spearman_scores": spearman(ours["scores"], ref_scores),
            "within_0.5pct": float(np.mean(np.abs(d - ref) <= tol)),
            "bit_identical_printable": float(np.mean(d[ok].view(np.uint32) == ref[ok].view(np.uint32))),
            "max_abs_diff_m": float(np.max(np.abs(d - ref))),
            "oversize_agree": bool(np.array_equal(d == -100, ref == -100)),
            "top_k_same_order": bool(np.array_equal(ref_top, ours["top"])),
        },
        "clocks": clk,
    }
    if np.array_equal(ref_top, ours["top"]):
        h = ours["hdist"].reshape(K, H)
        out["parity"]["holdout_within_0.5pct"] = float(np.mean(np.abs(h - ref_hold) <= 0.005 * np.maximum(np.abs(ref_hold), 1.0)))
    return out


def run_reference(args, world, rank, pg):
    """CPU arm: the reference's algorithm on the host cores (its flight exists only as CUDA, so
    this is the oracle port), one bounded sample of the workload per step."""
    if rank != 0:
        return
    sys.path.insert(0, ORACLE)
    import oracle_py

    # the genomes of the workload, drawn by the oracle (bit-identical to std::mt19937 grand());
    # nothing of this repository's library runs on this arm
    genomes = oracle_py.grand(args.seed, args.pop)
    nthreads = os.cpu_count() or 1
    sample = min(args.cpu_planes, args.pop)
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(genomes, args, nthreads)
        if i >= args.warmup:
            vals.append(r["value"])
            secs.append(r["seconds"])
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(secs)) * 1e3, "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": "sample of the 100k x 12 generation: %d genomes x %d scenarios per step" %
                       (sample, args.nseeds), "pop": args.pop, "nseeds": args.nseeds, "max_steps": args.max_steps},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d genomes x %d scenarios" % (sample, args.nseeds)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_grads(pe, torch, eng, dev, flush, args):
    """grads/sec of pe_grad and of central finite differences on the same GPU (see module doc)."""
    pop, S, T = args.grad_pop, args.grad_seeds, args.grad_steps
    G = pe.random_genomes(4, pop)
    seeds = list(range(1, S + 1))
    d_g = torch.from_numpy(G).to(dev)
    grad = torch.empty(pop, 35, device=dev)
    obj = torch.empty(pop, device=dev)

    def timed(fn, warmup, reps):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    g_ms = timed(lambda: eng.grad(d_g, pop, seeds, grad, max_steps=T, checkpoint_every=args.grad_every, d_obj=obj),
                 3, 5)
    tm = eng.last_timing()
    g_launches = tm["launches"]
    g_phases = {"prepare_ms": tm["prepare_ms"], "forward_ms": tm["flight_ms"], "reverse_and_genome_ms": tm["scores_ms"]}
    lo, hi = pe.genome_bounds()

    def perturbed(n):
        P = np.repeat(G[:n, None, :], 70, axis=1)
        for j in range(35):
            h = 1e-4 * (hi[j] - lo[j])
            P[:, 2 * j, j] += h
            P[:, 2 * j + 1, j] -= h
        return torch.from_numpy(np.ascontiguousarray(P.reshape(-1, 35), np.float32)).to(dev)

    P = perturbed(pop)
    nP = P.shape[0]
    ob = torch.empty(nP, device=dev, dtype=torch.float64)
    dd = torch.empty(nP * S, device=dev)
    fd32_eval = timed(lambda: eng.eval_batch(P, nP, seeds, 0, T, d_dist=dd), 3, 3)
    # the same evaluation kernels reporting the smoothed landing distance, scores = pe_grad's objective
    seng = pe.Engine(dev.index or 0)
    seng.set_smooth_landing(True)
    sobj = torch.empty(nP, device=dev)
    fd32_smooth = timed(lambda: seng.eval_batch(P, nP, seeds, 0, T, d_dist=dd, d_scores=sobj), 3, 3)
    seng.close()
    # those differences as a gradient (step 1e-4 of each gene's range, as pe_grad's check uses)
    so = sobj.cpu().numpy().astype(np.float64).reshape(pop, 35, 2)
    Pn = P.cpu().numpy().reshape(pop, 35 * 2, 35)
    hstep = np.stack([Pn[:, 2 * j, j].astype(np.float64) - Pn[:, 2 * j + 1, j] for j in range(35)], axis=1)
    fd32_grad = np.where(hstep > 0, (so[:, :, 0] - so[:, :, 1]) / np.where(hstep > 0, hstep, 1.0), 0.0)
    fd32 = timed(lambda: eng.objective(P, nP, seeds, precision=32, max_steps=T, d_obj=ob), 3, 3)
    n64 = min(args.fd64_genomes, pop)
    P64 = perturbed(n64)
    fd64 = timed(lambda: eng.objective(P64, P64.shape[0], seeds, precision=64, max_steps=T, d_obj=ob), 1, 2)
    rate = pop / (g_ms / 1e3)
    fd = {"fp64_objective": {"grads_per_s": n64 / (fd64 / 1e3), "sample": "%d genomes x 70" % n64},
          "fp32_objective": {"grads_per_s": pop / (fd32 / 1e3), "sample": "%d genomes x 70" % pop},
          "fp32_evaluator": {"grads_per_s": pop / (fd32_eval / 1e3), "sample": "%d genomes x 70" % pop,
                             "note": "unsmoothed landing distance: its differences are not a gradient"},
          "fp32_evaluator_smoothed": {"grads_per_s": pop / (fd32_smooth / 1e3), "sample": "%d genomes x 70" % pop,
                                      "note": "the evaluation kernels (body frame, packed f32x2) with the smoothed "
                                              "landing distance and the device tail-aware score: the differences "
                                              "of pe_grad's objective by the fastest forward pass here"}}
    for v in fd.values():
        v["speedup_of_pe_grad"] = rate / v["grads_per_s"]
    acc = None
    if not args.no_grad_accuracy:
        acc = grad_accuracy(pe, torch, eng, G, seeds, T, {"pe_grad": grad.cpu().numpy(),
                                                          "fd32_evaluator_smoothed": fd32_grad}, dev)
    return {"metric": "grads/sec", "value": rate, "unit": "grads/s", "ms_per_call": g_ms, "dtype": "f32",
            "workload": "%d genomes (std::mt19937(4) grand()) x %d scenarios (env seeds 1..%d), %d steps, "
                        "checkpoint every %d steps" % (pop, S, S, T, args.grad_every),
            "l2": "256 MB write between timed calls", "gpu_launches_per_call": g_launches, "phases": g_phases,
            "finite_differences": fd,
            "accuracy": acc}


def grad_accuracy(pe, torch, eng, G, seeds, T, grads, dev):
    """Gradients of every genome of the gradient workload (pe_grad, and FP32 central differences of the
    fastest forward pass) against FP64 central differences of the same objective on the GPU
    (pe_objective 64), as the tests take them: per gene the Richardson value of the largest step pair
    whose two differences agree; errors per gene relative to max(|ref_j|, 1e-2 max_k |ref_k|), and
    norm-wise."""
    n = G.shape[0]
    lo, hi = pe.genome_bounds()
    pairs = ((1e-4, 5e-5), (2e-5, 1e-5), (4e-6, 2e-6), (1e-6, 5e-7), (3e-7, 1.5e-7))
    fr = tuple(f for pr in pairs for f in pr)
    P = np.repeat(G[:, None, :], 35 * len(fr) * 2, axis=1).reshape(n, 35, len(fr), 2, 35)
    for j in range(35):
        for q, f in enumerate(fr):
            h = f * (hi[j] - lo[j])
            P[:, j, q, 0, j] = (G[:, j] + h).astype(np.float32)
            P[:, j, q, 1, j] = (G[:, j] - h).astype(np.float32)
    flat = torch.from_numpy(np.ascontiguousarray(P.reshape(-1, 35))).to(dev)
    o = torch.empty(flat.shape[0], device=dev, dtype=torch.float64)
    t0 = time.perf_counter()
    eng.objective(flat, flat.shape[0], seeds, precision=64, max_steps=T, d_obj=o)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    o = o.cpu().numpy().reshape(n, 35, len(fr), 2)
    D = np.zeros((n, 35, len(fr)))
    for j in range(35):
        D[:, j, :] = (o[:, j, :, 0] - o[:, j, :, 1]) / (P[:, j, :, 0, j].astype(np.float64) - P[:, j, :, 1, j])
    # the largest pair whose two differences agree to 1e-4 decides a gene (as the tests do): smooth
    # at that scale; smaller pairs resolve genes next to an active-set switch
    last = D[:, :, -1]
    scale = np.maximum(np.abs(last), 1e-2 * np.abs(last).max(axis=1, keepdims=True))
    ref = last.copy()
    for k in range(len(pairs) - 1, -1, -1):
        a, b = D[:, :, 2 * k], D[:, :, 2 * k + 1]
        ref = np.where(np.abs(a - b) <= 1e-4 * scale, (4 * b - a) / 3, ref)
    live = np.abs(ref).max(axis=1) > 0  # printable genomes (oversize ones have zero gradient)
    ref = ref[live]
    floor = 1e-2 * np.abs(ref).max(axis=1, keepdims=True)
    out = {"genomes": int(live.sum()), "pairs": int(ref.size),
           "reference": "FP64 central differences on the GPU (pe_objective 64): per gene the Richardson value of "
                        "the largest step pair, from (1e-4, 5e-5) of the gene range down to (3e-7, 1.5e-7), whose two "
                        "differences agree to 1e-4; %.1f s" % secs}
    for name, g in grads.items():
        g = np.asarray(g, np.float64)[live]
        gene = np.abs(g - ref) / np.maximum(np.abs(ref), floor)
        norm = np.linalg.norm(g - ref, axis=1) / np.linalg.norm(ref, axis=1)
        out[name] = {"per_gene_above_1e-3": float((gene >= 1e-3).mean()), "per_gene_max": float(gene.max()),
                     "per_gene_median": float(np.median(gene)),
                     "normwise_above_1e-3": float((norm >= 1e-3).mean()), "normwise_max": float(norm.max()),
                     "normwise_median": float(np.median(norm))}
    return out


def measure_configs(pe, torch, dev, flush, ref_cuda=True):
    """Throughput of the 1,024 x 8 and 8,192 x 8 evaluations (see module doc); median of 5 timed
    calls after 2 untimed ones, L2 flushed before each.  Beside them, host to host: this build's
    pe_evaluate_population (median of 5) and the reference's own CUDA build on the same genomes and
    seeds (oracle/ref_cuda_runner's eval mode: genomes H2D, k_prepare, per seed 12 synced 600-step
    k_sim launches + D2H, as gpu_prepare / gpu_sim run; median of 3 runs, clocks sampled), with the
    parity of its distances and scores."""
    import tempfile

    exe, ptx, why = ref_cuda_runner() if ref_cuda else (None, None, "--no-ref-cuda")
    out = {}
    S = 8
    for name, pop, seed in (("pop1024_x8", 1024, 0), ("pop8192_x8", 8192, 1)):
        g = torch.from_numpy(pe.random_genomes(seed, pop)).to(dev)
        seeds = [seed * S + s + 1 for s in range(S)]
        dist = torch.empty(pop * S, device=dev)
        steps = torch.empty(pop * S, dtype=torch.int32, device=dev)
        scores = torch.empty(pop, device=dev)
        row = {"workload": "%d genomes std::mt19937(%d) grand() x %d scenarios (env seeds %d..%d, vary 0), "
                           "7200 steps, scores on the device" % (pop, seed, S, seeds[0], seeds[-1])}
        shapes = [("one_launch", dict(use_graph=1)), ("chunks_600_graph", dict(chunk=600, use_graph=1))]
        shapes.append(("autotuned", None))
        for shape, kw in shapes:
            e = pe.Engine(dev.index or 0)
            if kw is None:  # the autotuner's pick for this batch, replayed from a graph
                e.autotune(g, pop, seeds, 0, 7200)
                e.set_config(use_graph=1)
            else:
                e.set_config(**kw)
            for _ in range(2):
                e.eval_batch(g, pop, seeds, 0, 7200, dist, steps, scores)
            torch.cuda.synchronize()
            plane_s = float(steps.sum().item()) / 600.0
            ms = []
            for _ in range(5):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                e.eval_batch(g, pop, seeds, 0, 7200, dist, steps, scores)
                b.record()
                torch.cuda.synchronize()
                ms.append(a.elapsed_time(b))
            med = sorted(ms)[len(ms) // 2]
            row[shape] = {"value": plane_s / (med / 1e3), "unit": UNIT, "ms": med, "launches": e.last_timing()["launches"],
                          "engine": e.config.as_dict()}
            e.close()
        row["plane_seconds"] = plane_s
        # host to host: this build from host buffers, then the reference build
        g_host = g.cpu().numpy()
        e = pe.Engine(dev.index or 0)
        for _ in range(2):
            mine = e.evaluate_population(g_host, seeds, max_steps=7200)
        walls = []
        for _ in range(5):
            t0 = time.perf_counter()
            mine = e.evaluate_population(g_host, seeds, max_steps=7200)
            walls.append(time.perf_counter() - t0)
        e.close()
        h2h = sorted(walls)[len(walls) // 2]
        row["host_to_host"] = {"value": plane_s / h2h, "unit": UNIT, "ms": h2h * 1e3,
                               "engine": "pe_evaluate_population, default shape, pageable numpy buffers"}
        if why:
            row["ref_cuda"] = {"unavailable": why}
        else:
            with tempfile.TemporaryDirectory() as tmp:
                gpath = os.path.join(tmp, "genomes.bin")
                np.ascontiguousarray(g_host, np.float32).tofile(gpath)
                clocks = Clocks(dev.index or 0)
                clocks.start()
                secs, ref, err = [], None, None
                for _ in range(3):
                    r = subprocess.run([exe, ptx, "eval", gpath, str(pop), "0", tmp] + [str(x) for x in seeds],
                                       capture_output=True, text=True)
                    if r.returncode != 0:
                        err = (r.stderr or r.stdout).strip()[-300:]
                        break
                    t = open(os.path.join(tmp, "timing.txt")).read().split()
                    secs.append(float(t[t.index("prepare_s") + 1]) + float(t[t.index("sim_s") + 1]))
                    ref = np.fromfile(os.path.join(tmp, "fitness.bin"), np.float32)
                clk = clocks.stop()
            if err:
                row["ref_cuda"] = {"unavailable": "reference runner failed: %s" % err}
            else:
                med = sorted(secs)[len(secs) // 2]
                d = mine["dist"]
                tol = 0.005 * np.maximum(np.abs(ref), 1.0)
                row["ref_cuda"] = {
                    "value": plane_s / med, "unit": UNIT, "seconds": secs,
                    "what": "the reference's k_prepare/k_sim as gpu_prepare/gpu_sim run them, host to host",
                    "ratio_host_to_host": med / h2h,
                    "parity": {"spearman_scores": spearman(mine["scores"], tail_scores(ref, S)),
                               "within_0.5pct": float(np.mean(np.abs(d - ref) <= tol)),
                               "oversize_agree": bool(np.array_equal(d == -100, ref == -100))},
                    "clocks": clk}
        out[name] = row
    return out


def measure_hybrid(eng, ga_seeds):
    """Plain device GA vs GA + Adam polish on the same GPU (see module doc), once per GA seed; the
    statistics over seeds (mean, sample sd) of each arm and of the paired differences."""
    common = dict(pop=16384, gens=30, nseeds=8, max_steps=7200, holdout=128, holdout_base=100003,
                  audit=4096, audit_base=9001)
    arms = (("plain", {}), ("hybrid", dict(polish_top=64, polish_steps=8, polish_lr=1e-2)))
    out = {"workload": "pop 16384 x 8 scenarios (training seeds gen*8+s+1), 30 generations, GA seeds %s; top 8 on a "
                       "128-scenario holdout (100003 + i*7919) each generation; best-ever audited on 4096 "
                       "scenarios (9001 + i*7919)" % ",".join(str(x) for x in ga_seeds),
           "max_steps": 7200, "ga_seeds": list(ga_seeds), "runs": []}
    for seed in ga_seeds:
        runs = {}
        for name, kw in arms:
            res, hist = eng.evolve(seed=seed, **common, **kw)
            runs[name] = (res, hist)
        target = runs["plain"][0]["best_holdout"]
        t_plain = runs["plain"][0]["gpu_seconds"]
        row = {"seed": seed}
        for name, (res, hist) in runs.items():
            best = np.maximum.accumulate(hist[:, 1])
            hit = np.flatnonzero(best >= target)
            at_plain_time = best[np.flatnonzero(hist[:, 4] <= t_plain)]
            row[name] = {"audit_score": res["audit_score"], "best_holdout": res["best_holdout"],
                         "gpu_seconds": res["gpu_seconds"], "grad_calls": res["grad_calls"],
                         "best_holdout_per_gpu_second": res["best_holdout"] / res["gpu_seconds"],
                         "gpu_seconds_to_plain_best_holdout": float(hist[hit[0], 4]) if hit.size else None,
                         "best_holdout_within_plain_gpu_seconds": float(at_plain_time[-1]) if at_plain_time.size else None}
        out["runs"].append(row)

    def stats(vals):
        v = np.array([x for x in vals if x is not None], np.float64)
        return {"mean": float(v.mean()) if v.size else None, "sd": float(v.std(ddof=1)) if v.size > 1 else None,
                "n": int(v.size)}

    for name, _ in arms:
        out[name] = {k: stats([r[name][k] for r in out["runs"]]) for k in
                     ("audit_score", "best_holdout", "gpu_seconds", "best_holdout_per_gpu_second",
                      "gpu_seconds_to_plain_best_holdout", "best_holdout_within_plain_gpu_seconds")}
    out["paired_difference_hybrid_minus_plain"] = {
        k: stats([r["hybrid"][k] - r["plain"][k] for r in out["runs"]])
        for k in ("audit_score", "best_holdout", "best_holdout_per_gpu_second")}
    out["paired_difference_hybrid_minus_plain"]["best_holdout_at_equal_gpu_seconds"] = stats(
        [r["hybrid"]["best_holdout_within_plain_gpu_seconds"] - r["plain"]["best_holdout"]
         if r["hybrid"]["best_holdout_within_plain_gpu_seconds"] is not None else None for r in out["runs"]])
    out["paired_difference_hybrid_minus_plain"]["speedup_to_plain_best"] = stats(
        [r["plain"]["gpu_seconds_to_plain_best_holdout"] / r["hybrid"]["gpu_seconds_to_plain_best_holdout"]
         if r["hybrid"]["gpu_seconds_to_plain_best_holdout"] else None for r in out["runs"]])
    return out


def run_gpu(args, world, rank, local, pg):
    import torch

    sys.path.insert(0, PKG)
    import pe

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pop, S, K = args.pop, args.nseeds, args.topk
    seeds, hseeds = training_seeds(args), holdout_seeds(args)
    # weak scaling: every rank flies its own population of `pop` genomes
    genomes = pe.random_genomes(rank_genome_seed(args, rank), pop)
    d_g = torch.from_numpy(genomes).to(dev)
    d_dist = torch.empty(pop * S, dtype=torch.float32, device=dev)
    d_steps = torch.empty(pop * S, dtype=torch.int32, device=dev)
    d_scores = torch.empty(pop, dtype=torch.float32, device=dev)
    d_top = torch.empty(K, 35, dtype=torch.float32, device=dev)
    d_hdist = torch.empty(K * len(hseeds), dtype=torch.float32, device=dev)
    d_hsteps = torch.empty(K * len(hseeds), dtype=torch.int32, device=dev)
    d_hscores = torch.empty(K, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    eng = pe.Engine(local)
    heng = pe.Engine(local)
    tuned = None
    if not args.no_autotune:
        tuned = eng.autotune(d_g, pop, seeds, 0, args.max_steps).as_dict()
    eng.set_config(use_graph=0 if args.no_graph else 1)
    heng.set_config(use_graph=0 if args.no_graph else 1)

    d_topi = torch.empty(K, dtype=torch.int32, device=dev)

    def generation():
        eng.eval_batch(d_g, pop, seeds, 0, args.max_steps, d_dist, d_steps, d_scores)
        pe.select_top(d_g, d_scores, pop, K, d_top, d_topi)
        heng.eval_batch(d_top, K, hseeds, 0, args.max_steps, d_hdist, d_hsteps, d_hscores)

    for _ in range(args.warmup):
        generation()
    torch.cuda.synchronize()
    # numerator: integrated steps (deterministic, identical every step)
    steps_main = int(d_steps.sum().item())
    steps_hold = int(d_hsteps.sum().item())
    plane_s_per_gen = (steps_main + steps_hold) / 600.0
    # algorithmic FLOPs of the flight kernel (per generation)
    nt = torch.empty(pop, dtype=torch.int32, device=dev)
    eng.plane_table(pop, d_nt=nt)
    nt_f = nt.to(torch.float64).repeat_interleave(S)
    hnt = torch.empty(K, dtype=torch.int32, device=dev)
    heng.plane_table(K, d_nt=hnt)
    hnt_f = hnt.to(torch.float64).repeat_interleave(len(hseeds))

    def gen_flops(per_panel, per_step):
        main = (d_steps.to(torch.float64) * (per_panel * nt_f + per_step)).sum().item()
        hold = (d_hsteps.to(torch.float64) * (per_panel * hnt_f + per_step)).sum().item()
        return float(main + hold)

    flops_gen = gen_flops(FLOP_PER_PANEL_STEP, FLOP_PER_STEP)
    flops_gen_body = gen_flops(FLOP_PER_PANEL_STEP_BODY, FLOP_PER_STEP_BODY)

    clocks = Clocks(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    flight_ms, launches = 0.0, 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record()
        generation()
        ev[i][1].record()
        tm, th = eng.last_timing(), heng.last_timing()
        flight_ms += tm["flight_ms"] + th["flight_ms"]
        launches += tm["launches"] + th["launches"] + 2  # prepare, flights, scores; top-8 select + gather
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = max_over_ranks(sum(step_ms) / 1e3, pg, dev)
    plane_s_job = sum_over_ranks(plane_s_per_gen, pg, dev)
    value = job_value(plane_s_job, args.steps, dev_s)

    # end to end through the host-buffer entry point (pinned host memory, copies included)
    h_g = torch.from_numpy(genomes).pin_memory()
    h_dist = torch.empty(pop * S, dtype=torch.float32).pin_memory()
    h_scores = torch.empty(pop, dtype=torch.float32).pin_memory()
    h_top = torch.empty(K, 35, dtype=torch.float32).pin_memory()
    h_hdist = torch.empty(K * len(hseeds), dtype=torch.float32).pin_memory()
    h_hscores = torch.empty(K, dtype=torch.float32).pin_memory()
    L = pe.LIB
    sp = np.asarray(seeds, np.int32)
    hsp = np.asarray(hseeds, np.int32)

    def generation_e2e():
        pe._check(L.pe_evaluate_population(eng.h, h_g.data_ptr(), pop, sp.ctypes.data, S, 0, args.max_steps,
                                           h_dist.data_ptr(), None, h_scores.data_ptr()))
        h_top.numpy()[:] = genomes[top_k_host(h_scores.numpy(), K)]
        pe._check(L.pe_evaluate_population(heng.h, h_top.data_ptr(), K, hsp.ctypes.data, len(hseeds), 0,
                                           args.max_steps, h_hdist.data_ptr(), None, h_hscores.data_ptr()))

    generation_e2e()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        generation_e2e()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t1, pg, dev)
    e2e_value = job_value(plane_s_job, args.steps, e2e_s)
    h2d = pop * 35 * 4 + K * 35 * 4
    d2h = pop * S * 4 + pop * 4 + K * len(hseeds) * 4 + K * 4

    if rank != 0:
        return
    peak = pe.fp32_peak_tflops(local)
    achieved = flops_gen * args.steps / (flight_ms / 1e3) / 1e12
    achieved_body = flops_gen_body * args.steps / (flight_ms / 1e3) / 1e12
    # DRAM bytes of the main flight launch: the per-flight figure of a 16k x 12 ncu capture (equal to
    # the algorithmic bytes: panels once per plane, state and distance per flight) times pop x S
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_flight_traffic.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile))["dram_bytes_per_flight"] * pop * S
    cpu = cpu_baseline(genomes, args)
    one = cpu_baseline(genomes, argparse.Namespace(**{**vars(args), "cpu_planes": args.cpu_planes_1core}), nthreads=1)
    cpu["one_core"] = {"value": one["value"], "sample": one["sample"]}
    ours = {"plane_s_per_gen": plane_s_per_gen, "value": value, "e2e_value": e2e_value,
            "dist": d_dist.cpu().numpy(), "scores": d_scores.cpu().numpy(), "top": d_topi.cpu().numpy(),
            "hdist": d_hdist.cpu().numpy()}
    ref_cuda = None if args.no_ref_cuda else measure_ref_cuda(args, genomes, ours, local)
    grads = None if args.no_grads else measure_grads(pe, torch, eng, dev, flush, args)
    hybrid = None if args.no_hybrid else measure_hybrid(heng, [int(x) for x in args.hybrid_seeds.split(",")])
    configs = None if args.no_configs else measure_configs(pe, torch, dev, flush, ref_cuda=not args.no_ref_cuda)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "generation at scale: %d genomes x %d scenarios (env seeds %d..%d, vary 0) + top-%d x "
                               "%d holdout (seeds %d + i*7919), max %d steps" %
                               (pop, S, seeds[0], seeds[-1], K, len(hseeds), args.holdout_base, args.max_steps),
                   "pop": pop, "nseeds": S, "holdout": len(hseeds), "max_steps": args.max_steps,
                   "genomes": "std::mt19937(%d) grand()" % args.seed,
                   "l2": "inputs larger than L2 (packed panels %.2f GB) and a 256 MB write between steps" %
                         (float(nt.sum().item()) * 32 / 1e9),
                   "engine": eng.config.as_dict(), "autotuned": tuned, "parallelism": "replicas" if world > 1 else "1 GPU"},
        "plane_seconds_per_step": plane_s_per_gen,
        "nominal_plane_seconds_per_step": (pop * S + K * len(hseeds)) * args.max_steps / 600.0,
        "roofline": {"bound": "fp32", "kernel": "k_flight", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": "profiles/k_flight_fast_pop16k_x12.md, scaled per flight to the main launch",
                     "peak_source": "measured FP32 FMA probe (pe_fp32_peak_probe), same process",
                     "flop_per_panel_step": FLOP_PER_PANEL_STEP, "flop_per_step": FLOP_PER_STEP,
                     "flop_source": "the reference step's per-plane-step count (128 nt + 300, FMA = 2)",
                     "formulation_count": {"flop_per_panel_step": FLOP_PER_PANEL_STEP_BODY,
                                           "flop_per_step": FLOP_PER_STEP_BODY, "achieved": achieved_body,
                                           "frac": achieved_body / peak,
                                           "note": "the body-frame formulation's own count: the print-warped "
                                                   "normal staged once per flight, not re-evaluated per step"},
                     "flight_ms_per_step": flight_ms / args.steps},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "ref_cuda": ref_cuda,
        "grads": grads,
        "hybrid": hybrid,
        "configs": configs,
        "clocks": clk,
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_gpu(args, world, rank, local, pg)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
