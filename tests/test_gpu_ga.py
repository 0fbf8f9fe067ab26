"""The device GA (pe_topk, pe_ga_step, pe_evolve).

pe_ga_step is checked against a numpy restatement of its operators (those of the reference's
run_ga, src/sim.cu:472-489) driven by the same counter-based SplitMix64 stream: uniform draws, selections and elites are
exact; fresh draws, blends and Gaussian mutations are compared to 1e-5 of a gene's range (the
device computes log and cos in fast math and may fuse a multiply-add).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


class _Stream:
    def __init__(self, seed, gen, child):
        self.key = _mix64(_mix64(seed) ^ ((gen << 32) | child))
        self.n = 0

    def u01(self):
        r = _mix64(self.key ^ ((self.n * 0xD1B54A32D192ED03) & M64))
        self.n += 1
        return np.float32(r >> 40) * np.float32(1.0 / 16777216.0)

    def normal(self):
        u1 = np.float32(1.0) - self.u01()
        u2 = self.u01()
        return np.float32(np.sqrt(-2.0 * np.log(np.float64(u1))) * np.cos(np.pi * 2.0 * np.float64(u2)))


def _ga_step_np(G, score, gen, gens, seed, lo, hi):
    pop = len(G)
    elite = pop // 64
    order = sorted(range(pop), key=lambda i: (-score[i], i))
    nxt = np.zeros_like(G)
    nxt[:elite] = G[order[:elite]]
    f32 = np.float32
    for i in range(elite, pop):
        r = _Stream(seed, gen, i)
        if r.u01() < f32(0.05):
            nxt[i] = [min(hi[j], max(lo[j], lo[j] + r.u01() * (hi[j] - lo[j]))) for j in range(35)]
            continue

        def tourn():
            b = min(int(r.u01() * f32(pop)), pop - 1)
            for _ in range(3):
                c = min(int(r.u01() * f32(pop)), pop - 1)
                if score[c] > score[b]:
                    b = c
            return b

        pa, pc = G[tourn()], G[tourn()]
        anneal = f32(1.0) - f32(0.6) * f32(gen) / f32(gens)
        for j in range(35):
            a = f32(-0.1) + f32(1.2) * r.u01()
            v = pa[j] * a + pc[j] * (f32(1) - a)
            if r.u01() < f32(0.25):
                v += r.normal() * f32(0.08) * (hi[j] - lo[j]) * anneal
            nxt[i, j] = min(hi[j], max(lo[j], v))
    return nxt


def test_topk_matches_numpy(cuda, pe):
    torch = cuda
    rng = np.random.default_rng(3)
    for n, k in ((1, 1), (100, 7), (5000, 256), (100000, 4096), (4096, 4096)):
        s = rng.integers(0, 50, n).astype(np.float32)  # many ties
        s[rng.integers(0, n, max(1, n // 50))] = np.nan
        d = torch.from_numpy(s).cuda()
        idx = torch.empty(k, dtype=torch.int32, device="cuda")
        top = torch.empty(k, device="cuda")
        pe.topk(d, n, k, idx, top)
        torch.cuda.synchronize()
        key = np.where(np.isnan(s), -np.inf, s)
        want = sorted(range(n), key=lambda i: (-key[i], np.isnan(s[i]), i))[:k]
        np.testing.assert_array_equal(idx.cpu().numpy(), want)
    with pytest.raises(pe.PEError):
        pe.topk(d, n, 4097, idx)
    # top-k + gather
    G = rng.normal(size=(n, 35)).astype(np.float32)
    d_g = torch.from_numpy(G).cuda()
    top = torch.empty(16, 35, device="cuda")
    ti = torch.empty(16, dtype=torch.int32, device="cuda")
    pe.select_top(d_g, d, n, 16, top, ti)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ti.cpu().numpy(), want[:16])
    np.testing.assert_array_equal(top.cpu().numpy(), G[want[:16]])


def test_ga_step_matches_restatement(cuda, pe, oracle):
    torch = cuda
    lo, hi = oracle.genome_bounds()
    G = oracle.grand(21, 256)
    rng = np.random.default_rng(5)
    score = rng.normal(5, 2, 256).astype(np.float32)
    score[rng.integers(0, 256, 30)] = -100.0
    d_g = torch.from_numpy(G).cuda()
    d_s = torch.from_numpy(score).cuda()
    d_n = torch.empty_like(d_g)
    for gen, seed in ((0, 5), (7, 5), (3, 123456789)):
        pe.ga_step(d_g, d_s, 256, gen, 30, seed, d_n)
        torch.cuda.synchronize()
        got = d_n.cpu().numpy()
        want = _ga_step_np(G, score, gen, 30, seed, lo, hi)
        np.testing.assert_array_equal(got[:4], want[:4])  # elites, best first
        assert (got >= lo).all() and (got <= hi).all()
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-5 * float((hi - lo).max()))
        pe.ga_step(d_g, d_s, 256, gen, 30, seed, d_n)  # deterministic
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_n.cpu().numpy(), got)
    with pytest.raises(pe.PEError):
        pe.ga_step(d_g, d_s, 256, 0, 30, 5, d_g)  # aliased output


def test_evolve_plain_and_hybrid(cuda, pe, engine):
    common = dict(pop=256, gens=4, nseeds=4, seed=5, max_steps=2400, holdout=32, audit=64)
    res_p, hist_p = engine.evolve(**common)
    res_h, hist_h = engine.evolve(polish_top=16, polish_steps=2, polish_lr=1e-2, **common)
    for res, hist in ((res_p, hist_p), (res_h, hist_h)):
        assert 0 <= res["best_gen"] < 4 and np.isfinite(res["best_holdout"]) and res["gpu_seconds"] > 0
        assert hist.shape == (4, 5) and np.isfinite(hist).all()
        assert (np.diff(hist[:, 4]) > 0).all() and hist[-1, 4] <= res["gpu_seconds"] + 1e-6
        assert res["best_holdout"] == hist[:, 1].max()
        # the audit is the best-ever genome's tail-aware score over audit_base + i * 7919
        out = engine.evaluate_population(res["best_genome"][None], [9001 + i * 7919 for i in range(64)],
                                         max_steps=2400, want_dist=False, want_steps=False)
        assert out["scores"][0] == res["audit_score"]
    assert res_p["grad_calls"] == 0 and res_h["grad_calls"] == 4 * 2
