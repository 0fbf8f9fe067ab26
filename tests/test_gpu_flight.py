"""GPU release / single steps / whole flights against the oracle.

Tolerances (floating point, FP32 fast-math device path vs FP32 host oracle and FP64 re-run):
  * teacher-forced step, aerodynamic force:  |F_gpu - F_64| <= 1e-5 max(|F_64|, m g)
  * teacher-forced step, aerodynamic torque: |T_gpu - T_64| <= 1e-5 max(|T_64|, chord m g)
    (m g, the plane's weight, is the force scale of a glide: a spinning release makes |F| a small
    difference of large panel forces, and torques cancel about the CG)
  * release state: 1e-5 relative per vector
  * whole flights (chaotic over ~10^3 steps): >= 90 % of printable flights within 0.5 % of the
    oracle's distance, and the tail-aware score ranking at Spearman >= 0.99 on 128 planes
Exact: oversize -> -100 with 0 steps, NaN state -> -10, the max_steps cut.
"""
import numpy as np
import pytest

from gpu_helpers import dev, eval_gpu, spearman, state_from_oracle

pytestmark = pytest.mark.gpu


def _rel(a, b, floor=1e-30):
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), floor)


def test_release_matches_oracle(cuda, any_engine, oracle):
    engine = any_engine
    torch = cuda
    G = oracle.grand(31, 96)
    seeds = [5, 900001]
    for vary in (0, 1):
        eval_gpu(torch, engine, G, seeds, vary=vary, max_steps=1, scores=False)
        st = torch.empty(len(G) * len(seeds), 16, dtype=torch.float32, device="cuda")
        engine.debug_release(len(G), seeds, vary, st)
        torch.cuda.synchronize()
        st = st.cpu().numpy()
        pre = oracle.Prepared(G)
        for p in np.where(pre.nt > 0)[0]:
            for s, seed in enumerate(seeds):
                r = pre.release(p, oracle.env_seed(seed, p, vary))
                g = st[p * len(seeds) + s]
                for sl in (slice(0, 3), slice(3, 7), slice(7, 10), slice(10, 13)):
                    assert _rel(g[sl], r[sl], 1e-6) <= 1e-5, (p, s, sl, g[sl], r[sl])


def test_teacher_forced_forces_within_1e5(cuda, any_engine, oracle):
    engine = any_engine
    torch = cuda
    G = oracle.grand(41, 48)
    seeds = [7, 8]
    S = len(seeds)
    pre32, pre64 = oracle.Prepared(G, 32), oracle.Prepared(G, 64)
    live = [p for p in range(len(G)) if pre32.nt[p] > 0][:24]
    # oracle trajectories: states at these step indices
    probe_steps = [0, 1, 7, 60, 250, 599, 600, 601]
    traj = {}
    for p in live:
        for s, seed in enumerate(seeds):
            st = pre32.release(p, seed)
            for k in range(max(probe_steps) + 1):
                if k > 0 and k % 600 == 0:  # the clock restart of a whole flight
                    st[13] = np.float32(k) * (np.float32(1.0) / np.float32(600.0))
                if k in probe_steps:
                    traj[(p, s, k)] = st.copy()
                st, _ = pre32.step(p, seed, st, k)
                if st[14]:
                    break
    eval_gpu(torch, engine, G, seeds, max_steps=1, scores=False)
    n = len(G) * S
    worst_f = worst_t = 0.0
    worst_f32 = 0.0
    checked = 0
    pure_f, pure_t = [], []  # |dF| / |F| and |dtau| / |tau| with no floor
    for k in probe_steps:
        sin = np.zeros((n, 16), np.float32)
        have = np.zeros(n, bool)
        for (p, s, kk), st in traj.items():
            if kk == k:
                sin[p * S + s] = state_from_oracle(st, k)
                have[p * S + s] = True
        if not have.any():
            continue
        d_in = dev(torch, sin)
        d_out = torch.empty_like(d_in)
        FT = torch.empty(n, 6, dtype=torch.float32, device="cuda")
        done = torch.empty(n, dtype=torch.int32, device="cuda")
        fit = torch.empty(n, dtype=torch.float32, device="cuda")
        for lanes in ((32, 16) if engine.config.formulation == 1 else (32,)):
            engine.debug_step(len(G), seeds, 0, 7200, d_in, d_out, FT, done, fit, k, lanes=lanes)
            torch.cuda.synchronize()
            ft = FT.cpu().numpy()
            for f in np.where(have)[0]:
                p, s = divmod(int(f), S)
                st = traj[(p, s, k)]
                _, ft64 = pre64.step(p, seeds[s], st.astype(np.float64), k)
                _, ft32 = pre32.step(p, seeds[s], st, k)
                weight = float(pre64.mp[p, 0]) * 9.81
                fs = max(np.linalg.norm(ft64[:3]), weight)
                ef = np.linalg.norm(ft[f, :3] - ft64[:3]) / fs
                et = np.linalg.norm(ft[f, 3:] - ft64[3:]) / max(np.linalg.norm(ft64[3:]), G[p, 1] * weight)
                worst_f, worst_t = max(worst_f, ef), max(worst_t, et)
                worst_f32 = max(worst_f32, np.linalg.norm(ft32[:3] - ft64[:3]) / fs)
                pure_f.append(np.linalg.norm(ft[f, :3] - ft64[:3]) / max(np.linalg.norm(ft64[:3]), 1e-30))
                pure_t.append(np.linalg.norm(ft[f, 3:] - ft64[3:]) / max(np.linalg.norm(ft64[3:]), 1e-30))
                checked += 1
    assert checked > 100
    pure_f, pure_t = np.array(pure_f), np.array(pure_t)
    print("teacher-forced (formulation %d): GPU vs FP64 force %.2e torque %.2e (host FP32 force %.2e)" %
          (engine.config.formulation, worst_f, worst_t, worst_f32))
    print("  pure relative, %d steps: |dF|/|F| median %.2e p99 %.2e max %.2e, share > 1e-5 %.4f; "
          "|dtau|/|tau| median %.2e p99 %.2e max %.2e, share > 1e-5 %.4f" %
          (len(pure_f), np.median(pure_f), np.quantile(pure_f, 0.99), pure_f.max(), np.mean(pure_f > 1e-5),
           np.median(pure_t), np.quantile(pure_t, 0.99), pure_t.max(), np.mean(pure_t > 1e-5)))
    assert worst_f <= 1e-5 and worst_t <= 1e-5


def test_flights_match_oracle(cuda, any_engine, oracle):
    engine = any_engine
    torch = cuda
    G = oracle.grand(2, 128)
    seeds = [25, 26, 27, 28]
    out = eval_gpu(torch, engine, G, seeds)
    rd, rs = oracle.eval_batch(G, seeds)
    printable = rs > 0
    assert np.array_equal(out["steps"] > 0, printable)
    assert np.all(out["dist"][~printable] == -100.0) and np.all(out["steps"][~printable] == 0)
    d, r = out["dist"][printable], rd[printable]
    within = np.abs(d - r) <= 0.005 * np.maximum(np.abs(r), 1.0)
    same_steps = np.mean(out["steps"][printable] == rs[printable])
    rho = spearman(out["scores"], oracle.robust_scores(rd, len(G), len(seeds)))
    print("formulation %d: flights within 0.5%%: %.4f  same step count: %.4f  spearman: %.5f" %
          (engine.config.formulation, within.mean(), same_steps, rho))
    assert within.mean() >= 0.90
    assert rho >= 0.99
    # the device score of the device distances is the oracle's score of the same numbers
    assert np.array_equal(out["scores"], oracle.robust_scores(out["dist"], len(G), len(seeds)))


def test_fault_paths_nan_oversize_and_cut(cuda, any_engine, oracle):
    engine = any_engine
    torch = cuda
    G = oracle.grand(5, 64)
    pre = oracle.Prepared(G)
    ok = np.where(pre.nt > 0)[0]
    bad = G[ok[:2]].copy()
    bad[0, 11] = np.nan  # NaN ballast gene: printable mesh, NaN mass -> -10 (src/sim.cu:198-201)
    out = eval_gpu(torch, engine, np.concatenate([G, bad]), [3, 4])
    n = len(G)
    assert np.all(out["dist"][2 * n:2 * n + 2] == -10.0) and np.all(out["steps"][2 * n:2 * n + 2] == 1)
    over = np.where(pre.nt == 0)[0]
    for p in over:
        assert np.all(out["dist"][2 * p:2 * p + 2] == -100.0) and np.all(out["steps"][2 * p:2 * p + 2] == 0)
    # flights cut at max_steps are credited pos.x at step max_steps - 1
    cut = eval_gpu(torch, engine, G, [3], max_steps=40)
    rd, rs = oracle.eval_batch(G, [3], max_steps=40)
    assert np.array_equal(cut["steps"], rs)
    m = rs == 40
    assert m.any()
    assert np.all(np.abs(cut["dist"][m] - rd[m]) <= 1e-4 * np.maximum(np.abs(rd[m]), 1.0))


def test_argument_errors(cuda, engine, pe):
    torch = cuda
    g = torch.zeros(4, 35, device="cuda")
    with pytest.raises(pe.PEError) as e:
        engine.eval_batch(g, 0, [1])
    assert e.value.code == pe.PE_EINVAL
    with pytest.raises(pe.PEError):
        engine.eval_batch(g, 4, [], max_steps=10)
    with pytest.raises(pe.PEError):
        engine.eval_batch(g, 4, [1], max_steps=7201)
    with pytest.raises(pe.PEError):
        engine.set_config(lanes=8)


def test_allocation_failure_is_a_status(cuda, pe, oracle):
    """A call whose buffers cannot be allocated returns an error status from the allocation, before
    any kernel runs, and the context stays usable: pe_grad of 65,536 genomes x 256 scenarios with a
    checkpoint every step asks for ~7.7 PB of checkpoints.  (The largest evaluation, PE_MAX_POP
    planes, fits a GB300; above it pop is PE_EINVAL before any allocation.)"""
    torch = cuda
    e = pe.Engine(0)
    pop = 65536
    g = torch.zeros(pop, 35, device="cuda")
    gr = torch.empty(pop, 35, device="cuda")
    with pytest.raises(pe.PEError) as err:
        e.grad(g, pop, list(range(1, 257)), gr, max_steps=7200, checkpoint_every=1)
    assert err.value.code == pe.PE_ECUDA and "memory" in str(err.value)
    with pytest.raises(pe.PEError) as err:
        e.eval_batch(g, pe.MAX_POP + 1, [1], 0, 7200)
    assert err.value.code == pe.PE_EINVAL
    e.close()
    G = oracle.grand(5, 16)
    e2 = pe.Engine(0)
    out = e2.evaluate_population(G, [3, 4], max_steps=1200)
    ref, _ = oracle.eval_batch(G, [3, 4], vary=0, max_steps=1200)
    assert np.array_equal(out["dist"] == -100, ref == -100)
    e2.close()


def test_smooth_landing_distances(cuda, pe, oracle):
    """pe_engine_set_smooth_landing: flights ended by ground contact report the z = 0 crossing between
    their last two states, as the oracle's smoothed flight (fly_smooth) and pe_grad's objective do;
    every other ending, the step counts and the printability are those of the plain evaluation."""
    torch = cuda
    G = oracle.grand(23, 96)
    seeds = [11, 12, 13]
    eng = pe.Engine(0)
    plain = eval_gpu(torch, eng, G, seeds)
    eng.set_smooth_landing(True)
    sm = eval_gpu(torch, eng, G, seeds)
    assert np.array_equal(sm["steps"], plain["steps"])
    pre = oracle.Prepared(G, 32)
    ref = np.array([pre.fly_smooth(p, s)[0] for p in range(len(G)) for s in seeds], np.float32)
    kinds = np.array([pre.fly_smooth(p, s)[2] for p in range(len(G)) for s in seeds])
    assert np.array_equal(sm["dist"] == -100, ref == -100)
    within = np.abs(sm["dist"] - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0)
    assert within.mean() >= 0.99, within.mean()
    ground = kinds == 1
    # the interpolated point lies between the last two states: within one step of flight (|v| <= 60 m/s)
    assert np.all(np.abs(plain["dist"][ground] - sm["dist"][ground]) <= 60.0 / 600.0 + 1e-5)
    assert np.array_equal(sm["dist"][~ground], plain["dist"][~ground])
    # the tail-aware score of the smoothed distances is pe_grad's objective (FP32 model, IEEE math)
    g = dev(torch, G.astype(np.float32))
    obj = torch.empty(len(G), device="cuda")
    gr = torch.empty(len(G), 35, device="cuda")
    eng.grad(g, len(G), seeds, gr, max_steps=7200, d_obj=obj)
    torch.cuda.synchronize()
    o = obj.cpu().numpy()
    ok = np.abs(sm["scores"] - o) <= 0.005 * np.maximum(np.abs(o), 1.0)
    assert ok.mean() >= 0.97, ok.mean()
    eng.set_config(formulation=0, lanes=32, reg_cap=0)
    with pytest.raises(pe.PEError) as e:
        eval_gpu(torch, eng, G[:4], seeds)
    assert e.value.code == pe.PE_ENOTSUP
    eng.close()
