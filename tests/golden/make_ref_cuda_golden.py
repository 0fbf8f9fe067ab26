"""Record golden vectors from the reference's own CUDA build on a GPU.

Step 1, on a GPU host (the PTX of the reference's src/sim.cu must already sit in
oracle/_ref/ref_sim.ptx, built by oracle/build.py where the reference tree exists):
    python tests/golden/make_ref_cuda_golden.py run <out_dir>
runs oracle/ref_cuda_runner (the reference's k_prepare / k_sim, driven like gpu_prepare /
gpu_sim) on seeded synthetic populations and writes the raw outputs to <out_dir>.
Step 2, anywhere:
    python tests/golden/make_ref_cuda_golden.py pack <out_dir>
packs them into tests/golden/ref_cuda_golden.npz:
  c1_genomes [512][35] grand(0); c1_seeds [8] = 1..8 (the GA's seeds for generation 0, vary 0)
  c1_fitness [512][8], c1_nt [512], c1_mp [512][20], c1_pc / c1_pn [256][900][4]
  ev_genomes [64][35] grand(9001)[:64]; ev_seed 9001, vary 1: ev_fitness [64]
  rel_states [64][15]   release states (k_sim with step0 = 0, nsteps = 0), seed 33, vary 1
  st_in [64][15], st_out [64][15], st_fit [64]   one resumed step (step0 = 1, nsteps = 1)
  rec_genomes [16][35] grand(14)[:16]; rec_params (seed 5, vary 1, rec_every 30, rec_cap 240),
  rec_spread 0.5: rec [16][240][8] (pos xyz, q wxyz, alive; NaN where never written), rec_fitness
  timing lines of each run
Two more sets, recorded the same way (`run2 <out_dir>` on the GPU host, then `pack2 <out_dir>`):
  tests/golden/ref_cuda_c3_slice.npz  the first 10,000 genomes of the 100,000 x 12 generation
      (grand(2)[:10000], regenerated by the oracle's bit-exact draw) under env seeds 25..36, vary 0:
      fitness [10000][12]
  tests/golden/ref_cuda_traj.npz  teacher-forcing states: genomes grand(33)[:64], seed 33, vary 1;
      for k in TRAJ_STEPS the reference's state at step k (in [6][64][15]) and after one resumed
      step from it (out [6][64][15])
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle_py  # noqa: E402

obuild = oracle_py._build

PTX = os.path.join(ROOT, "oracle", "_ref", "ref_sim.ptx")
# the recorded run: genomes grand(14)[:16], seed 5, vary 1, a pose every 30 steps, 240 slots
# (the whole 7200-step horizon), launch grid spacing 0.5 m
REC = dict(pop=16, seed=5, vary=1, every=30, cap=240, spread=0.5)
OUT_NPZ = os.path.join(HERE, "ref_cuda_golden.npz")
C3_NPZ = os.path.join(HERE, "ref_cuda_c3_slice.npz")
TRAJ_NPZ = os.path.join(HERE, "ref_cuda_traj.npz")
C3_SLICE = dict(pop=10000, seed=2, nseeds=12)
TRAJ = dict(pop=64, genome_seed=33, seed=33, vary=1)
TRAJ_STEPS = (1, 7, 60, 599, 600, 601)


def _runner():
    return obuild.build_ref_cuda_runner()


def run(out):
    os.makedirs(out, exist_ok=True)
    exe = _runner()
    # C1-like: 512 genomes, the GA's training seeds of generation 0 (gen*S + s + 1, vary 0)
    g = oracle_py.grand(0, 512)
    g.tofile(os.path.join(out, "c1_genomes.bin"))
    d = os.path.join(out, "c1")
    os.makedirs(d, exist_ok=True)
    subprocess.run([exe, PTX, "eval", os.path.join(out, "c1_genomes.bin"), "512", "0", d] +
                   [str(s) for s in range(1, 9)], check=True)
    # evaluate-style: the same genome replicated, vary 1 (src/sim.cu:260-267)
    ge = np.repeat(oracle_py.grand(9001, 1), 64, axis=0)
    ge.tofile(os.path.join(out, "ev_genomes.bin"))
    d = os.path.join(out, "ev")
    os.makedirs(d, exist_ok=True)
    subprocess.run([exe, PTX, "eval", os.path.join(out, "ev_genomes.bin"), "64", "1", d, "9001"], check=True)
    # release states and one resumed step
    gs = oracle_py.grand(33, 64)
    gs.tofile(os.path.join(out, "st_genomes.bin"))
    d = os.path.join(out, "rel")
    os.makedirs(d, exist_ok=True)
    subprocess.run([exe, PTX, "release", os.path.join(out, "st_genomes.bin"), "64", "1", "33", d], check=True)
    d2 = os.path.join(out, "step")
    os.makedirs(d2, exist_ok=True)
    subprocess.run([exe, PTX, "step", os.path.join(out, "st_genomes.bin"), "64", "1", "33",
                    os.path.join(d, "states.bin"), "1", "1", d2], check=True)
    # pose recording with the showcase launch grid, as render.cu drives gpu_sim
    gr = oracle_py.grand(14, REC["pop"])
    gr.tofile(os.path.join(out, "rec_genomes.bin"))
    d = os.path.join(out, "rec")
    os.makedirs(d, exist_ok=True)
    subprocess.run([exe, PTX, "record", os.path.join(out, "rec_genomes.bin"), str(REC["pop"]), str(REC["vary"]),
                    str(REC["seed"]), str(REC["every"]), str(REC["cap"]), repr(REC["spread"]), d], check=True)


def pack(out):
    f = lambda *p: os.path.join(out, *p)  # noqa: E731
    c1g = np.fromfile(f("c1_genomes.bin"), np.float32).reshape(512, 35)
    evg = np.fromfile(f("ev_genomes.bin"), np.float32).reshape(64, 35)
    stg = np.fromfile(f("st_genomes.bin"), np.float32).reshape(64, 35)
    arrays = dict(
        c1_genomes=c1g, c1_seeds=np.arange(1, 9, dtype=np.int32),
        c1_fitness=np.fromfile(f("c1", "fitness.bin"), np.float32).reshape(512, 8),
        c1_nt=np.fromfile(f("c1", "nt.bin"), np.int32),
        c1_mp=np.fromfile(f("c1", "mp.bin"), np.float32).reshape(512, 20),
        c1_pc=np.fromfile(f("c1", "pc.bin"), np.float32).reshape(256, 900, 4)[:64],
        c1_pn=np.fromfile(f("c1", "pn.bin"), np.float32).reshape(256, 900, 4)[:64],
        ev_genomes=evg, ev_seed=np.int32(9001),
        ev_fitness=np.fromfile(f("ev", "fitness.bin"), np.float32).reshape(64),
        st_genomes=stg, st_seed=np.int32(33),
        rel_states=np.fromfile(f("rel", "states.bin"), np.float32).reshape(64, 15),
        st_out=np.fromfile(f("step", "states.bin"), np.float32).reshape(64, 15),
        st_fit=np.fromfile(f("step", "fitness.bin"), np.float32).reshape(64),
        timing=np.array([open(f(k, "timing.txt")).read().strip() for k in ("c1", "ev")]),
    )
    if os.path.exists(f("rec", "rec.bin")):
        arrays.update(
            rec_genomes=np.fromfile(f("rec_genomes.bin"), np.float32).reshape(REC["pop"], 35),
            rec_params=np.array([REC["seed"], REC["vary"], REC["every"], REC["cap"]], np.int32),
            rec_spread=np.float32(REC["spread"]),
            rec=np.fromfile(f("rec", "rec.bin"), np.float32).reshape(REC["pop"], REC["cap"], 8),
            rec_fitness=np.fromfile(f("rec", "fitness.bin"), np.float32).reshape(REC["pop"]),
        )
    np.savez_compressed(OUT_NPZ, **arrays)
    print("wrote", OUT_NPZ, os.path.getsize(OUT_NPZ), "bytes")


def run2(out):
    os.makedirs(out, exist_ok=True)
    exe = _runner()
    c = C3_SLICE
    g = oracle_py.grand(c["seed"], c["pop"])
    g.tofile(os.path.join(out, "c3_genomes.bin"))
    d = os.path.join(out, "c3")
    os.makedirs(d, exist_ok=True)
    seeds = [c["seed"] * c["nseeds"] + s + 1 for s in range(c["nseeds"])]
    subprocess.run([exe, PTX, "eval", os.path.join(out, "c3_genomes.bin"), str(c["pop"]), "0", d] +
                   [str(s) for s in seeds], check=True)
    t = TRAJ
    gt = oracle_py.grand(t["genome_seed"], t["pop"])
    gt.tofile(os.path.join(out, "traj_genomes.bin"))
    d = os.path.join(out, "traj")
    os.makedirs(d, exist_ok=True)
    subprocess.run([exe, PTX, "traj", os.path.join(out, "traj_genomes.bin"), str(t["pop"]), str(t["vary"]),
                    str(t["seed"]), d] + [str(k) for k in TRAJ_STEPS], check=True)


def pack2(out):
    f = lambda *p: os.path.join(out, *p)  # noqa: E731
    c = C3_SLICE
    np.savez_compressed(C3_NPZ, fitness=np.fromfile(f("c3", "fitness.bin"), np.float32).reshape(c["pop"], c["nseeds"]),
                        genome_seed=np.int32(c["seed"]),
                        seeds=np.array([c["seed"] * c["nseeds"] + s + 1 for s in range(c["nseeds"])], np.int32),
                        timing=np.array(open(f("c3", "timing.txt")).read().strip()))
    t = TRAJ
    ins = np.stack([np.fromfile(f("traj", "in_%d.bin" % k), np.float32).reshape(t["pop"], 15) for k in TRAJ_STEPS])
    outs = np.stack([np.fromfile(f("traj", "out_%d.bin" % k), np.float32).reshape(t["pop"], 15) for k in TRAJ_STEPS])
    np.savez_compressed(TRAJ_NPZ, steps=np.array(TRAJ_STEPS, np.int32), genome_seed=np.int32(t["genome_seed"]),
                        seed=np.int32(t["seed"]), vary=np.int32(t["vary"]), state_in=ins, state_out=outs)
    for p in (C3_NPZ, TRAJ_NPZ):
        print("wrote", p, os.path.getsize(p), "bytes")


def full(out, pop=100000, seed=2, nseeds=12):
    """Reference build vs this engine on one full generation (default: 100k x 12, seeds 25..36):
    the reference's wall time and a parity summary (summary.json) small enough to commit."""
    import json
    import time

    pop, seed, nseeds = int(pop), int(seed), int(nseeds)
    os.makedirs(out, exist_ok=True)
    exe = _runner()
    g = oracle_py.grand(seed, pop)
    gpath = os.path.join(out, "genomes.bin")
    g.tofile(gpath)
    seeds = [seed * nseeds + s + 1 for s in range(nseeds)]
    d = os.path.join(out, "ref")
    os.makedirs(d, exist_ok=True)
    t0 = time.perf_counter()
    subprocess.run([exe, PTX, "eval", gpath, str(pop), "0", d] + [str(s) for s in seeds], check=True)
    ref_wall = time.perf_counter() - t0
    ref = np.fromfile(os.path.join(d, "fitness.bin"), np.float32)
    sys.path.insert(0, os.path.join(ROOT, "planes-rl_gb300"))
    import pe
    from scipy.stats import spearmanr
    rs = oracle_py.robust_scores(ref, pop, nseeds)
    ok = ref > -100
    summary = {
        "workload": "%d genomes grand(%d) x %d scenarios (seeds %d..%d, vary 0)" % (pop, seed, nseeds, seeds[0], seeds[-1]),
        "ref_timing": open(os.path.join(d, "timing.txt")).read().strip(),
        "ref_wall_s_incl_process_and_jit": ref_wall,
        "printable_flights": int(ok.sum()),
    }
    for form in (0, 1):
        eng = pe.Engine(0)  # formulation 1: the engine's default shape
        if form == 0:
            eng.set_config(formulation=0, reg_cap=0, lanes=32)
        mine = eng.evaluate_population(g, seeds)
        t1 = time.perf_counter()
        mine = eng.evaluate_population(g, seeds)
        wall = time.perf_counter() - t1
        summary["formulation_%d" % form] = {
            "engine_wall_s_host_to_host": wall,
            "bit_identical_fraction": float(np.mean(mine["dist"].view(np.uint32) == ref.view(np.uint32))),
            "bit_identical_fraction_printable": float(np.mean(mine["dist"][ok].view(np.uint32) == ref[ok].view(np.uint32))),
            "within_0.5pct_fraction": float(np.mean(np.abs(mine["dist"] - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0))),
            "max_abs_diff_m": float(np.max(np.abs(mine["dist"] - ref))),
            "oversize_agree": bool(np.array_equal(mine["dist"] == -100, ref == -100)),
            "spearman_scores": float(spearmanr(mine["scores"], rs).statistic),
            "scores_bit_identical_fraction": float(np.mean(mine["scores"].view(np.uint32) == rs.view(np.uint32))),
            "plane_seconds": float(mine["steps"].sum()) / 600.0,
        }
        eng.close()
    json.dump(summary, open(os.path.join(out, "summary.json"), "w"), indent=1)
    print(json.dumps(summary, indent=1))


if __name__ == "__main__":
    {"run": run, "pack": pack, "run2": run2, "pack2": pack2, "full": full}[sys.argv[1]](*sys.argv[2:])
