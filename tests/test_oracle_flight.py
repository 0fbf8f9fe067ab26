"""Host-side checks of the oracle's flight and fitness code (no GPU)."""
import numpy as np
import pytest


def f32(x):
    return np.float32(x)


def reference_scores(samples, pop, S):
    """src/sim.cu:340-357 written out step by step in float32 (known-answer form)."""
    out = np.zeros(pop, np.float32)
    tail = (S + 3) // 4
    for i in range(pop):
        row = samples[i * S:(i + 1) * S].astype(np.float32)
        mean = f32(0)
        for x in row:
            mean = f32(mean + f32(x / f32(S)))
        srt = np.sort(row)
        cvar = f32(0)
        for s in range(tail):
            cvar = f32(cvar + f32(srt[s] / f32(tail)))
        out[i] = f32(f32(f32(f32(0.65) * mean) + f32(f32(0.25) * cvar)) + f32(f32(0.10) * srt[0]))
    return out


@pytest.mark.parametrize("S", [1, 2, 3, 4, 5, 8, 12, 13, 128])
def test_robust_scores_known_answer(oracle, S):
    rng = np.random.default_rng(S)
    pop = 37
    samples = rng.normal(6, 4, pop * S).astype(np.float32)
    samples[rng.random(pop * S) < 0.1] = -100.0
    samples[rng.random(pop * S) < 0.05] = -10.0
    samples[1::7] = samples[0:-1:7][: samples[1::7].size]  # ties
    got = oracle.robust_scores(samples, pop, S)
    want = reference_scores(samples, pop, S)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_robust_scores_hand_example(oracle):
    # S = 4: tail = 1; mean = 2.5, cvar25 = worst = 1 -> 0.65*2.5 + 0.25*1 + 0.10*1
    s = np.array([4, 1, 3, 2], np.float32)
    got = oracle.robust_scores(s, 1, 4)[0]
    assert got == f32(f32(f32(0.65) * f32(2.5)) + f32(0.25)) + f32(f32(0.10) * f32(1))
    assert abs(got - 1.975) < 1e-6


def test_oversize_and_nan_paths(oracle):
    g = oracle.grand(5, 64)
    pre = oracle.Prepared(g)
    oversize = np.where(pre.nt == 0)[0]
    assert oversize.size > 0
    dist, steps = pre.eval([11, 12], vary=0, max_steps=600)
    for p in oversize:
        assert np.all(dist[p * 2:(p + 1) * 2] == -100.0) and np.all(steps[p * 2:(p + 1) * 2] == 0)
    # a NaN nose-ballast gene keeps the mesh printable but poisons mass -> fitness -10
    bad = g[~(pre.nt == 0)][:1].copy()
    bad[0, 11] = np.nan
    d, n = oracle.eval_batch(bad, [3], max_steps=600)
    assert d[0] == -10.0 and n[0] == 1


def test_max_steps_credit_distance(oracle):
    """A flight cut at max_steps is credited pos.x at step max_steps - 1 (src/sim.cu:202-203)."""
    g = oracle.grand(8, 32)
    pre = oracle.Prepared(g)
    p = int(np.where(pre.nt > 0)[0][0])
    fit, n, st = pre.fly(p, 21, max_steps=40)
    assert n == 40 and fit == st[0] and st[14] == 1


def test_chunk_clock_restart(oracle):
    """A whole flight equals single steps with the clock reset to 600 * dt at step 600, the
    restart of every 600-step launch of the reference (src/sim.cu:113, 241-244)."""
    g = oracle.grand(3, 64)
    pre = oracle.Prepared(g)
    dt = np.float32(1.0) / np.float32(600.0)
    for p in np.where(pre.nt > 0)[0]:
        fit, n, final = pre.fly(p, 5, max_steps=605)
        if n < 605:
            continue  # landed before the restart
        st = pre.release(p, 5)
        for k in range(605):
            if k == 600:
                assert st[13] != np.float32(600) * dt  # the accumulated clock drifted
                st[13] = np.float32(600) * dt
            st, _ = pre.step(p, 5, st, k, max_steps=605)
        assert np.array_equal(st.view(np.uint32), final.view(np.uint32))
        return
    pytest.skip("no flight of this sample outlived 605 steps")


def test_fp32_fp64_teacher_forced_forces(oracle):
    """One step from identical states: FP32 vs FP64 aerodynamic sums agree to ~1e-6."""
    g = oracle.grand(12, 24)
    p32, p64 = oracle.Prepared(g, 32), oracle.Prepared(g, 64)
    worst = 0.0
    for p in np.where(p32.nt > 0)[0][:8]:
        st = p32.release(p, 77)
        for k in range(0, 120):
            nxt, ft32 = p32.step(p, 77, st, k)
            _, ft64 = p64.step(p, 77, st.astype(np.float64), k)
            for a, b in ((ft32[:3], ft64[:3]), (ft32[3:], ft64[3:])):
                worst = max(worst, float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-3)))
            if nxt[14]:
                break
            st = nxt
    assert worst < 1e-4, worst


def test_eval_threads_deterministic(oracle):
    g = oracle.grand(21, 24)
    a = oracle.eval_batch(g, [1, 2, 3], nthreads=1)
    b = oracle.eval_batch(g, [1, 2, 3], nthreads=4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _audit_f32(d):
    """src/sim.cu:250-256 and 291-309 written out in numpy float32 (every operation rounded)."""
    f = np.float32
    s = np.sort(np.asarray(d, f))
    n = s.size

    def pct(q):
        x = f(q) * f(n - 1)
        a, b = int(np.floor(x)), int(np.ceil(x))
        t = f(x - f(a))
        return f(s[a] * f(f(1) - t)) + f(s[b] * t)

    mean, sq = f(0), f(0)
    for x in s:
        mean = f(mean + f(x / f(n)))
        sq = f(sq + f(f(x * x) / f(n)))
    sd = f(np.sqrt(max(f(0), f(sq - f(mean * mean)))))
    tail = max(1, n // 10)
    cvar = f(0)
    for x in s[:tail]:
        cvar = f(cvar + f(x / f(tail)))
    return np.array([s[0], pct(.05), pct(.10), pct(.25), pct(.50), mean, sd, pct(.75), pct(.90), pct(.95), s[-1],
                     cvar, np.sum(s < 0)], f)


@pytest.mark.parametrize("n", [1, 2, 7, 10, 11, 1000, 4099])
def test_audit_stats_against_float32_restatement(oracle, n):
    """The oracle's audit statistics (or_audit_stats) against an independent float32 restatement:
    bit for bit, with ties, failures (negative distances) and -100 rows."""
    rng = np.random.default_rng(n)
    d = rng.normal(6.0, 4.0, n).astype(np.float32)
    d[rng.integers(0, n, max(1, n // 7))] = -100.0
    d[rng.integers(0, n, max(1, n // 5))] = 3.25
    got, want = oracle.audit_stats(d), _audit_f32(d)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert got[0] == d.min() and got[10] == d.max() and got[12] == np.sum(d < 0)


def test_oracle_flights_match_reference_cuda_build(oracle):
    """The oracle's flight restatement (float) pinned directly to the reference's own CUDA build: the
    512 genomes x 8 seeds of the golden vectors (grand(0), env seeds 1..8, vary 0), recorded on a
    GB300 from the reference's k_prepare / k_sim.  At least 99 % of flights within 0.5 % (or 5 mm
    below 1 m), oversize exact, Spearman of the tail-aware scores >= 0.999."""
    import os

    from scipy.stats import spearmanr

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cuda_golden.npz")
    gold = np.load(path)
    G, seeds, ref = gold["c1_genomes"], [int(s) for s in gold["c1_seeds"]], gold["c1_fitness"].reshape(-1)
    dist, steps = oracle.eval_batch(G, seeds)
    assert np.array_equal(dist == -100, ref == -100) and np.all(steps[ref == -100] == 0)
    within = np.mean(np.abs(dist - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0))
    pr = ref > -100
    same = np.mean(dist[pr].view(np.uint32) == ref[pr].view(np.uint32))
    rho = spearmanr(oracle.robust_scores(dist, len(G), len(seeds)), oracle.robust_scores(ref, len(G), len(seeds))).statistic
    print("oracle vs reference CUDA build, %d flights: within 0.5%% %.5f, bit-identical (printable) %.4f, spearman %.9f"
          % (dist.size, within, same, rho))
    assert within >= 0.99 and rho >= 0.999
