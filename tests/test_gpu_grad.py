"""pe_grad on the GPU: d(smoothed tail-aware objective)/d(genome) against the FP64 model and the
oracle's FP64 central finite differences.

The tolerance is the one the path is specified to, 1e-3 relative to FP64 central differences at
a step of 1e-4 of each gene's range, applied two ways: norm-wise, |g - ref| / |ref| <= 1e-3, and
per gene, |g_j - ref_j| <= 1e-3 max(|ref_j|, 1e-2 max_k |ref_k|).  Over large populations
(gpu_helpers.check_grad_population) the norm-wise bar must hold for 99 % of the genomes and the
per-gene bar for 99.5 % of the pairs (both 1e-2 for all): where the objective is strongly curved
next to an active-set switch, the FP32 trajectory's rounding moves the gradient by a few 1e-3.  The per-gene floor keeps genes
whose derivative is ~1e-4 of the largest on the gradient's scale: on flights of 1,100+ steps the
FP32 trajectory's own rounding, amplified by the flight, moves those by ~1e-7 of the largest
component (the host FP32 run of the same model does the same).  The differences are Richardson-extrapolated from that step and half of it,
(4 D(h/2) - D(h)) / 3: some genes (the outer dihedral, for one) have third derivatives large
enough that D(1e-4) alone is ~0.7% off the derivative it estimates.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = list(range(25, 33))
GRAD_TOL = 1e-3


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _host_model(lib, oracle, g, seeds, max_steps, K=60):
    """The same model and adjoint in double on the host (pe_grad_model.h)."""
    S = len(seeds)
    scen = np.stack([oracle.scenario_desc(int(s), prec=64) for s in seeds]).astype(np.float64)
    sd = np.asarray(seeds, np.int32)
    J, gr, d = np.zeros(1), np.zeros(35), np.zeros(S)
    kind, st = np.zeros(S, np.int32), np.zeros(S, np.int32)
    lib.pgh_objective_grad(_p(np.ascontiguousarray(g, np.float32)), _p(scen), _p(sd), S, max_steps, K, _p(J), _p(gr),
                           _p(d), _p(kind), _p(st))
    return J[0], gr, d


def _central(oracle, g, j, h, seeds, max_steps):
    gp, gm = g.copy(), g.copy()
    gp[j] = np.float32(g[j] + h)
    gm[j] = np.float32(g[j] - h)
    jp = oracle.smooth_objective(gp, seeds, max_steps)[0]
    jm = oracle.smooth_objective(gm, seeds, max_steps)[0]
    return (jp - jm) / (float(gp[j]) - float(gm[j]))


def _fd(oracle, g, seeds, max_steps, rel_h=1e-4):
    lo, hi = oracle.genome_bounds()
    out = np.zeros(35)
    for j in range(35):
        h = rel_h * (hi[j] - lo[j])
        out[j] = (4 * _central(oracle, g, j, h / 2, seeds, max_steps) - _central(oracle, g, j, h, seeds, max_steps)) / 3
    return out


def _rel_err(g, ref, floor_frac=1e-2):
    floor = floor_frac * np.abs(ref).max()
    return np.abs(g - ref) / np.maximum(np.abs(ref), floor)


def _check_grad(g, ref, tag=""):
    norm = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    err = _rel_err(g, ref)
    strict = _rel_err(g, ref, 1e-3)
    print(f"{tag} norm-wise {norm:.2e}  per-gene {err.max():.2e} (gene {int(err.argmax())})  "
          f"per-gene with 1e-3 floor {strict.max():.2e}")
    assert norm < GRAD_TOL, (tag, norm)
    assert err.max() < GRAD_TOL, (tag, err.max(), int(err.argmax()))


def _run(cuda, engine, G, seeds, vary=0, max_steps=3600, K=60):
    torch = cuda
    pop = G.shape[0]
    d_g = torch.from_numpy(np.ascontiguousarray(G, np.float32)).cuda()
    grad = torch.empty(pop, 35, device="cuda")
    obj = torch.empty(pop, device="cuda")
    dist = torch.empty(pop * len(seeds), device="cuda")
    engine.grad(d_g, pop, seeds, grad, vary=vary, max_steps=max_steps, checkpoint_every=K, d_obj=obj, d_dist=dist)
    torch.cuda.synchronize()
    return obj.cpu().numpy().astype(np.float64), grad.cpu().numpy().astype(np.float64), dist.cpu().numpy()


@pytest.fixture(scope="module")
def population(oracle):
    G = oracle.grand(4, 256)
    pre = oracle.Prepared(G, prec=32)
    printable = np.flatnonzero(pre.nt > 0)
    return G, printable


def test_grad_matches_oracle_finite_differences(cuda, engine, oracle, population):
    G, printable = population
    sel = G[printable[:3]]
    obj, grad, dist = _run(cuda, engine, sel, SEEDS, max_steps=3600)
    for i in range(sel.shape[0]):
        fd = _fd(oracle, sel[i], SEEDS, 3600)
        Jo, do = oracle.smooth_objective(sel[i], SEEDS, 3600)
        assert obj[i] == pytest.approx(Jo, rel=1e-4)
        np.testing.assert_allclose(dist[i * 8:(i + 1) * 8], do, rtol=5e-3)
        _check_grad(grad[i], fd, f"genome {i} vs FD:")


def test_grad_matches_fp64_model_across_population(cuda, engine, grad_host, oracle, population):
    """32 genomes, printable and oversize mixed: objective and gradient against the host FP64
    run of the same model (which itself equals the oracle's finite differences)."""
    G, printable = population
    sel = G[:32]
    obj, grad, dist = _run(cuda, engine, sel, SEEDS, max_steps=3600)
    for i in range(sel.shape[0]):
        J, gr, d = _host_model(grad_host, oracle, sel[i], SEEDS, 3600)
        if J == -100:
            assert obj[i] == -100 and not grad[i].any()
            continue
        assert obj[i] == pytest.approx(J, rel=1e-4)
        _check_grad(grad[i], gr, f"genome {i} vs FP64 model:")


def test_grad_checkpoint_interval_and_vary(cuda, engine, population):
    """The checkpoint interval changes only the schedule of the recompute: the forward outputs are
    bit-identical, and the gradients agree to 1e-4 (the reverse rebuilds up to K steps from each
    checkpoint with this model's integrator on the forward's stored forces, so its states carry the
    rounding of two float implementations of one step over at most K steps)."""
    G, printable = population
    sel = G[printable[:16]]
    o60, g60, d60 = _run(cuda, engine, sel, SEEDS[:4], max_steps=2400, K=60)
    for K in (1, 7, 600):
        o, g, d = _run(cuda, engine, sel, SEEDS[:4], max_steps=2400, K=K)
        np.testing.assert_array_equal(d, d60)
        np.testing.assert_array_equal(o, o60)
        np.testing.assert_allclose(g, g60, rtol=1e-4, atol=1e-6 * np.abs(g60).max())
    # vary = 1: plane p flies env seeds seed + p * 7919, as in pe_eval_batch
    ov, gv, dv = _run(cuda, engine, sel[:4], [11], vary=1, max_steps=2400)
    for i in range(4):
        oi, gi, di = _run(cuda, engine, sel[i:i + 1], [11 + i * 7919], max_steps=2400)
        assert dv[i] == di[0]
        np.testing.assert_allclose(gv[i], gi[0], rtol=1e-6, atol=1e-7 * np.abs(gi).max())


def test_grad_horizon_flights_and_edge_sizes(cuda, engine, grad_host, oracle, population):
    G, printable = population
    sel = G[printable[:4]]
    obj, grad, dist = _run(cuda, engine, sel, SEEDS[:4], max_steps=150)
    for i in range(4):
        J, gr, d = _host_model(grad_host, oracle, sel[i], SEEDS[:4], 150)
        np.testing.assert_allclose(dist[i * 4:(i + 1) * 4], d, rtol=1e-4)
        _check_grad(grad[i], gr, f"horizon genome {i}:")
    # one seed, one genome; and the largest seed count
    o1, g1, d1 = _run(cuda, engine, sel[:1], [5], max_steps=1200)
    J, gr, d = _host_model(grad_host, oracle, sel[0], [5], 1200)
    _check_grad(g1[0], gr, "one seed:")
    o256, g256, d256 = _run(cuda, engine, sel[:2], list(range(256)), max_steps=600)
    assert np.isfinite(g256).all() and np.isfinite(o256).all()


def test_grad_rejects_bad_arguments(cuda, engine, pe, population):
    torch = cuda
    G, printable = population
    d_g = torch.from_numpy(np.ascontiguousarray(G[:2], np.float32)).cuda()
    grad = torch.empty(2, 35, device="cuda")
    with pytest.raises(pe.PEError):
        engine.grad(d_g, 2, list(range(257)), grad)
    with pytest.raises(pe.PEError):
        engine.grad(d_g, 2, [1], grad, checkpoint_every=601)
    with pytest.raises(pe.PEError):
        engine.grad(d_g, 2, [1], None)
    with pytest.raises(pe.PEError):
        engine.grad(d_g, 2, [1], grad, max_steps=7201)


def test_grad_torch_autograd(cuda, engine, pe, population):
    torch = cuda
    G, printable = population
    g = torch.from_numpy(np.ascontiguousarray(G[printable[:4]], np.float32)).cuda().requires_grad_(True)
    obj = pe.genome_objective(engine, g, SEEDS[:4], max_steps=1200)
    w = torch.tensor([1.0, -2.0, 0.5, 3.0], device="cuda")
    (obj * w).sum().backward()
    o, gr, d = _run(cuda, engine, G[printable[:4]], SEEDS[:4], max_steps=1200)
    np.testing.assert_allclose(obj.detach().cpu().numpy(), o, rtol=0, atol=0)
    np.testing.assert_allclose(g.grad.cpu().numpy(), gr * w.cpu().numpy()[:, None], rtol=1e-6)


# ---------------------------------------------------------------- pe_objective (forward only)
def _objective(cuda, engine, G, seeds, precision, max_steps=3600, vary=0):
    torch = cuda
    pop = G.shape[0]
    d_g = torch.from_numpy(np.ascontiguousarray(G, np.float32)).cuda()
    obj = torch.empty(pop, device="cuda", dtype=torch.float64)
    dist = torch.empty(pop * len(seeds), device="cuda", dtype=torch.float64)
    engine.objective(d_g, pop, seeds, precision=precision, vary=vary, max_steps=max_steps, d_obj=obj, d_dist=dist)
    torch.cuda.synchronize()
    return obj.cpu().numpy(), dist.cpu().numpy()


def test_objective_fp64_matches_oracle_and_fp32(cuda, engine, oracle, population):
    G, printable = population
    sel = G[:24]
    o64, d64 = _objective(cuda, engine, sel, SEEDS, 64)
    o32, d32 = _objective(cuda, engine, sel, SEEDS, 32)
    og, _, dg = _run(cuda, engine, sel, SEEDS, max_steps=3600)
    # The GPU draws each scenario in float (the evaluation path's draw) and widens it; the oracle's
    # FP64 run draws it in double.  That ~1e-8 relative difference of the inputs, carried through
    # a flight, bounds the agreement; it is the same for every perturbation of a genome, so it
    # does not enter finite differences.
    for i in range(sel.shape[0]):
        Jo, do = oracle.smooth_objective(sel[i], SEEDS, 3600)
        assert o64[i] == pytest.approx(Jo, rel=1e-6, abs=1e-5)
        np.testing.assert_allclose(d64[i * 8:(i + 1) * 8], do, rtol=1e-6, atol=1e-5)  # metres
    np.testing.assert_allclose(o32, o64, rtol=1e-4)
    np.testing.assert_allclose(og, o64, rtol=1e-4)  # pe_grad's own objective


def test_grad_matches_gpu_fp64_finite_differences(cuda, engine, oracle, population):
    """64 genomes: pe_grad against FP64 central differences computed on the GPU by pe_objective
    (which equals the oracle's FP64 objective, see above), Richardson-extrapolated from steps of
    1e-4 and 5e-5 of the gene's range, or from smaller pairs where that estimate has not converged
    because an active-set switch (a tail-quartile member, a clamp) lies within the step
    (gpu_helpers.fd64_per_gene).  How many genes needed the smaller steps is printed."""
    from gpu_helpers import check_grad_population, fd64_per_gene

    G, printable = population
    sel = G[printable[:64]]
    og, grad, _ = _run(cuda, engine, sel, SEEDS, max_steps=3600)
    lo, hi = oracle.genome_bounds()
    fd, levels = fd64_per_gene(cuda, engine, sel, SEEDS, 3600, lo, hi)
    print("genes decided by step pairs 1e-4, 2e-5, 4e-6, 1e-6, 3e-7 of the range, none:", levels.tolist())
    check_grad_population(grad, fd, "vs GPU FD64:")


def test_engine_destroy_frees_gradient_and_objective_buffers(cuda, pe):
    """Each cycle grows an engine's gradient (checkpoints, adjoints, ~120 MB at 1000 x 8 x 3600)
    and objective buffers, then destroys the engine: device free memory must come back."""
    torch = cuda
    pop, seeds = 1000, list(range(1, 9))
    d_g = torch.from_numpy(pe.random_genomes(9, pop)).cuda()
    grad = torch.empty(pop, 35, device="cuda")

    def cycle():
        eng = pe.Engine(0)
        eng.grad(d_g, pop, seeds, grad, max_steps=3600)
        eng.objective(d_g, pop, seeds, precision=64, max_steps=600)
        torch.cuda.synchronize()
        eng.close()

    cycle()  # module loading and the context's own first allocations
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        cycle()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < (32 << 20), (free0 - free1) / 2**20


def test_grad_stored_forces_match_panel_recompute(cuda, engine, population, monkeypatch):
    """The forward pass is the evaluation's packed body-frame kernel on this model's set-up; the
    reverse pass rebuilds each segment's states from its checkpoint with this model's integrator.
    By default it takes every step's body force and torque from the forward pass; with
    PE_GRAD_STORE_FORCES=0 it recomputes them with this model's panel pass.  The forward outputs
    (objectives, distances) are bit-identical either way; the two rebuilt trajectories differ by the
    rounding of two float implementations of the panel sums over at most K steps, and the gradients
    agree to 1e-4 norm-wise (checkpoint intervals 60 and 7, vary 0 and 1)."""
    G, printable = population
    sel = G[printable[:24]]
    for K, vary in ((60, 0), (7, 1)):
        want = _run(cuda, engine, sel, SEEDS[:4], max_steps=2400, K=K, vary=vary)
        monkeypatch.setenv("PE_GRAD_STORE_FORCES", "0")
        got = _run(cuda, engine, sel, SEEDS[:4], max_steps=2400, K=K, vary=vary)
        monkeypatch.delenv("PE_GRAD_STORE_FORCES")
        for i in (0, 2):  # objective, distances
            np.testing.assert_array_equal(np.asarray(got[i]).view(np.uint32), np.asarray(want[i]).view(np.uint32))
        g, w = np.asarray(got[1], np.float64), np.asarray(want[1], np.float64)
        norm = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-30)
        print("K %d vary %d: stored vs recomputed forces, gradient norm-wise max %.2e" % (K, vary, norm.max()))
        assert norm.max() <= 1e-4


def test_grad_forward_flies_the_evaluation_physics(cuda, engine, pe, population):
    """pe_grad's forward pass (the evaluation kernel on this model's IEEE set-up of each flight) lands
    where the evaluation kernels' smoothed landing does (pe_engine_set_smooth_landing), to rounding:
    distances within 0.5 % for at least 99 % of flights and the objective within 0.5 % of the
    smoothed tail-aware score, at the GA's small training seeds.  With large seeds (vary 1) the two
    models draw different gust scales: the evaluation, like the reference build, takes sinf of
    seed * 1.61803 with fast-math (a rough sine at 1e5-1e6 rad), the gradient model takes it in IEEE
    float; that case is printed, not asserted."""
    torch = cuda
    from gpu_helpers import eval_gpu
    G, printable = population
    sel = np.ascontiguousarray(G[:40], np.float32)
    for seeds, vary in ((SEEDS[:4], 0), ([9001], 1)):
        o, g, d = _run(cuda, engine, sel, seeds, vary=vary, max_steps=2400)
        ev = pe.Engine(0)
        ev.set_smooth_landing(True)
        out = eval_gpu(torch, ev, sel, seeds, vary=vary, max_steps=2400)
        ev.close()
        d = np.asarray(d).reshape(-1)
        ok = np.abs(d - out["dist"]) <= 0.005 * np.maximum(np.abs(out["dist"]), 1.0)
        oo = np.abs(np.asarray(o) - out["scores"]) <= 0.005 * np.maximum(np.abs(out["scores"]), 1.0)
        print("vary %d: distances within 0.5%% %.4f, objectives %.4f" % (vary, ok.mean(), oo.mean()))
        assert np.array_equal(d == -100, out["dist"] == -100)
        if vary == 0:
            assert ok.mean() >= 0.99 and oo.mean() >= 0.97


def test_grad_long_flight_pass_matches_the_batched_pass(cuda, engine, population):
    """A small batch (at most 4 flights per SM) sends its longest flights through the pipelined
    reverse pass (a block per flight: warp 1 rebuilding the next segment, warp 2 its step_pre and gust
    Jacobian, warp 0 only differentiating); a large batch does not.  The same 24 genomes alone (192
    flights) and inside the 256-genome population (2,048 flights) give the same objectives and
    distances bit for bit, and gradients that agree to 1e-5 norm-wise."""
    G, printable = population
    sel = printable[:24]
    o_s, g_s, d_s = _run(cuda, engine, G[sel], SEEDS, max_steps=3600)
    o_b, g_b, d_b = _run(cuda, engine, G, SEEDS, max_steps=3600)
    d_b = np.asarray(d_b).reshape(len(G), len(SEEDS))[sel].reshape(-1)
    np.testing.assert_array_equal(np.asarray(d_s).view(np.uint32), d_b.view(np.uint32))
    np.testing.assert_array_equal(np.asarray(o_s), np.asarray(o_b)[sel])
    g_b = np.asarray(g_b)[sel]
    norm = np.linalg.norm(np.asarray(g_s) - g_b, axis=1) / np.maximum(np.linalg.norm(g_b, axis=1), 1e-30)
    print("long-flight pass vs batched pass: gradient norm-wise max %.2e" % norm.max())
    assert norm.max() <= 1e-5


def test_grad_grouped_blocks(cuda, engine, population, monkeypatch):
    """With the stored forces the reverse pass runs the longest flights pipelined, the next ones a
    block each, and the rest two to a block, warp 0 carrying both integrator chains at once.  Which
    flights share a block changes nothing: with every flight in a block of its own
    (PE_GRAD_GROUP=1) objectives, distances and gradients are the same bit for bit.  Against the
    one-flight kernel (PE_GRAD_GROUP=0) objectives and distances are bit-identical and gradients
    agree to 1e-5 norm-wise: the grouped blocks have 3 warps, so each step's panel adjoints are
    summed over 96 threads instead of 128, in another order (measured: 1e-6).  Cases: the 256-genome
    population (2,048 flights, oversize ones included, an odd count sharing blocks), 101 genomes x 3
    scenarios with checkpoints every 7 steps and every 96 (the largest interval of the grouped and
    long-flight passes; above 60 the grouped pass runs without its rebuild pipeline), vary 1."""
    G, printable = population
    cases = [(G, SEEDS, 3600, 60, 0), (G[:101], SEEDS[:3], 2400, 7, 0), (G[:101], SEEDS[:3], 2400, 96, 0),
             (G[printable[:64]], [9001, 9002, 9003], 2400, 60, 1)]
    for Gc, seeds, max_steps, K, vary in cases:
        got = _run(cuda, engine, Gc, seeds, vary=vary, max_steps=max_steps, K=K)
        monkeypatch.setenv("PE_GRAD_GROUP", "1")
        single = _run(cuda, engine, Gc, seeds, vary=vary, max_steps=max_steps, K=K)
        monkeypatch.setenv("PE_GRAD_GROUP", "0")
        one = _run(cuda, engine, Gc, seeds, vary=vary, max_steps=max_steps, K=K)
        monkeypatch.delenv("PE_GRAD_GROUP")
        for w, g in zip(single, got):
            np.testing.assert_array_equal(np.asarray(g), np.asarray(w))
        for i in (0, 2):
            np.testing.assert_array_equal(np.asarray(got[i]), np.asarray(one[i]))
        g, w = np.asarray(got[1]), np.asarray(one[1])
        norm = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-30)
        print("%d x %d, K %d, vary %d: shared blocks bit-identical to single ones; vs the one-flight kernel "
              "%d genomes differ, norm-wise max %.2e" % (Gc.shape[0], len(seeds), K, vary, int((g != w).any(1).sum()),
                                                        norm.max()))
        assert norm.max() <= 1e-5
