"""The differentiable model behind pe_grad, on the CPU.

planes-rl_gb300/csrc/pe_grad_model.h is instantiated in double (and float) on the host and
checked against the oracle:
  * its mesh / mass properties / panels equal the oracle's FP64 prepare (src/common.h:124-365,
    src/sim.cu:25-49);
  * its smoothed landing distance equals the oracle's fly_smooth;
  * its reverse-mode flight adjoint + forward-mode genome contraction equals FP64 central finite
    differences of the oracle's tail-aware objective (src/sim.cu:340-357 weights) over the
    smoothed distance, gene by gene.
"""
import ctypes as C

import numpy as np
import pytest

D = np.float64
SEEDS = list(range(25, 33))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _plane(lib, g):
    m, I, com = np.zeros(1), np.zeros(6), np.zeros(3)
    c, A, n = np.zeros((344, 3)), np.zeros(344), np.zeros((344, 3))
    nt = np.zeros(1, np.int32)
    pr = lib.pgh_plane_data(_p(np.ascontiguousarray(g, np.float32)), _p(m), _p(I), _p(com), _p(c), _p(A), _p(n),
                            _p(nt))
    k = int(nt[0])
    return pr, m[0], I, com, c[:k], A[:k], n[:k]


def _flight(lib, sc, seed, m, I, c, A, n, max_steps, K=60):
    nt = len(A)
    kind, steps = np.zeros(1, np.int32), np.zeros(1, np.int32)
    Lm, LI, Lc, LA, Ln = np.zeros(1), np.zeros(6), np.zeros((nt, 3)), np.zeros(nt), np.zeros((nt, 3))
    d = lib.pgh_flight(_p(sc), seed, m, _p(np.ascontiguousarray(I)), nt, _p(np.ascontiguousarray(c)),
                       _p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(n)), max_steps, K, _p(kind), _p(steps),
                       _p(Lm), _p(LI), _p(Lc), _p(LA), _p(Ln))
    return d, int(kind[0]), int(steps[0]), Lm[0], LI, Lc, LA, Ln


def _objgrad(lib, oracle, g, seeds, max_steps, K=60, f32=False):
    S = len(seeds)
    scen = np.stack([oracle.scenario_desc(int(s), prec=32 if f32 else 64) for s in seeds]).astype(D)
    sd = np.asarray(seeds, np.int32)
    J, gr, d = np.zeros(1), np.zeros(35), np.zeros(S)
    kind, st = np.zeros(S, np.int32), np.zeros(S, np.int32)
    fn = lib.pgh_objective_grad_f32 if f32 else lib.pgh_objective_grad
    fn(_p(np.ascontiguousarray(g, np.float32)), _p(scen), _p(sd), S, max_steps, K, _p(J), _p(gr), _p(d), _p(kind),
       _p(st))
    return J[0], gr, d, kind, st


def _fd_genome(oracle, g, seeds, max_steps, genes, rel_h=1e-4):
    """FP64 central differences of the oracle's objective at a step of 1e-4 of each gene's range
    (normalized genome units); the step is the float32-representable
    difference of the perturbed genes (the oracle reads float32 genomes)."""
    lo, hi = oracle.genome_bounds()
    out = {}
    for j in genes:
        h = rel_h * (hi[j] - lo[j])
        gp, gm = g.copy(), g.copy()
        gp[j] = np.float32(g[j] + h)
        gm[j] = np.float32(g[j] - h)
        jp = oracle.smooth_objective(gp, seeds, max_steps)[0]
        jm = oracle.smooth_objective(gm, seeds, max_steps)[0]
        out[j] = (jp - jm) / (float(gp[j]) - float(gm[j]))
    return out


@pytest.fixture(scope="module")
def genomes(oracle):
    G = oracle.grand(2, 64)
    pre = oracle.Prepared(G, prec=64)
    return G, pre


def test_plane_data_matches_oracle_fp64(grad_host, genomes):
    G, pre = genomes
    for p in range(12):
        pr, m, I, com, c, A, n = _plane(grad_host, G[p])
        assert bool(pr) == bool(pre.nt[p] > 0)
        assert m == pytest.approx(pre.mp[p, 0], rel=1e-12)
        np.testing.assert_allclose(I, pre.mp[p, 5:11], rtol=0, atol=1e-9 * np.abs(pre.mp[p, 5:8]).max())
        np.testing.assert_allclose(com, pre.mp[p, 2:5], rtol=0, atol=1e-8)
        if pr:
            k = len(A)
            np.testing.assert_allclose(c, pre.pc[p, :k, :3], rtol=0, atol=1e-8)
            np.testing.assert_allclose(A, pre.pc[p, :k, 3], rtol=1e-10, atol=1e-15)
            np.testing.assert_allclose(n, pre.pn[p, :k, :3], rtol=0, atol=1e-8)


def test_smooth_distance_matches_oracle_fp64(grad_host, oracle, genomes):
    G, pre = genomes
    planes = [p for p in range(64) if pre.nt[p] > 0][:3]
    for p in planes:
        _, m, I, _, c, A, n = _plane(grad_host, G[p])
        for seed in (25, 26, 27):
            sc = oracle.scenario_desc(seed, prec=64).astype(D)
            for max_steps in (7200, 150):
                d, kind, steps, *_ = _flight(grad_host, sc, seed, m, I, c, A, n, max_steps)
                do, so, ko = pre.fly_smooth(p, seed, max_steps)
                assert (kind, steps) == (ko, so)
                assert d == pytest.approx(do, rel=1e-6)


def test_flight_adjoint_matches_fd_on_plane_data(grad_host, oracle, genomes):
    """Adjoint of one flight's distance wrt mass, inertia and some panels, against central
    differences of the same double-precision forward."""
    G, pre = genomes
    p, seed = 2, 26
    _, m, I, _, c, A, n = _plane(grad_host, G[p])
    sc = oracle.scenario_desc(seed, prec=64).astype(D)
    for max_steps in (120, 7200):  # horizon-ended and landed
        d, kind, steps, Lm, LI, Lc, LA, Ln = _flight(grad_host, sc, seed, m, I, c, A, n, max_steps)
        assert kind == (2 if max_steps == 120 else 1)

        def f(m_=m, I_=I, c_=c, A_=A, n_=n):
            return _flight(grad_host, sc, seed, m_, I_, c_, A_, n_, max_steps)[0]

        h = 1e-6 * m
        assert Lm == pytest.approx((f(m_=m + h) - f(m_=m - h)) / (2 * h), rel=1e-5)
        hI = 1e-5 * I[:3].max()
        for q in range(6):
            Ip, Im = I.copy(), I.copy()
            Ip[q] += hI
            Im[q] -= hI
            assert LI[q] == pytest.approx((f(I_=Ip) - f(I_=Im)) / (2 * hI), rel=1e-5)
        for t in (0, 100, 170):
            for k in range(3):
                cp, cm = c.copy(), c.copy()
                cp[t, k] += 1e-7
                cm[t, k] -= 1e-7
                scale = np.abs(Lc).max()
                assert abs(Lc[t, k] - (f(c_=cp) - f(c_=cm)) / 2e-7) < 1e-4 * scale
            Ap, Am = A.copy(), A.copy()
            Ap[t] *= 1 + 1e-6
            Am[t] *= 1 - 1e-6
            assert LA[t] == pytest.approx((f(A_=Ap) - f(A_=Am)) / (2e-6 * A[t]), rel=1e-4)


@pytest.mark.parametrize("p", [0, 2])
def test_genome_gradient_matches_oracle_fd(grad_host, oracle, genomes, p):
    G, pre = genomes
    g = G[p].astype(np.float32)
    J, gr, d, kind, st = _objgrad(grad_host, oracle, g, SEEDS, 7200)
    Jo, do = oracle.smooth_objective(g, SEEDS, 7200)
    assert J == pytest.approx(Jo, rel=1e-7)
    assert (kind == 1).all()
    fd = _fd_genome(oracle, g, SEEDS, 7200, range(35))
    fdv = np.array([fd[j] for j in range(35)])
    floor = 1e-3 * np.abs(fdv).max()
    err = np.abs(gr - fdv) / np.maximum(np.abs(fdv), floor)
    assert err.max() < 1e-5, (err.max(), int(err.argmax()))
    # the same model in float (the GPU kernels' precision) stays within 1e-3 of the FP64 differences
    J32, gr32, *_ = _objgrad(grad_host, oracle, g, SEEDS, 7200, f32=True)
    assert J32 == pytest.approx(Jo, rel=1e-5)
    err32 = np.abs(gr32 - fdv) / np.maximum(np.abs(fdv), floor)
    assert err32.max() < 1e-3, (err32.max(), int(err32.argmax()))


def test_gradient_horizon_flights_and_oversize(grad_host, oracle, genomes):
    G, pre = genomes
    g = G[6].astype(np.float32)
    J, gr, d, kind, st = _objgrad(grad_host, oracle, g, SEEDS[:4], 150)
    assert (kind == 2).all() and (st == 150).all()
    fd = _fd_genome(oracle, g, SEEDS[:4], 150, [0, 1, 7, 21, 34])
    for j, v in fd.items():
        assert abs(gr[j] - v) <= 1e-5 * max(abs(v), 1e-3 * np.abs(gr).max())
    big = [p for p in range(64) if pre.nt[p] == 0][0]
    J, gr, d, kind, st = _objgrad(grad_host, oracle, G[big], SEEDS[:4], 7200)
    assert J == -100 and (d == -100).all() and not gr.any()
