"""Parity at the full sizes the path is measured on, through properties that do not depend on size.

* 100,000 genomes x 12 scenarios (the bench's generation, seeds 25..36, 7200 steps):
  - a random sample of 300 genomes against the oracle (FP32, the reference's arithmetic):
    distances within the path's bar (0.5 %, or 2 cm near zero), oversize exactly, ranking
    (Spearman of the tail-aware scores) >= 0.999;
  - permutation invariance: the same genomes in another order fly bit-identically;
  - the device's tail-aware scores equal the host reduction of its own distances, bit for bit.
* 256 genomes x 8 scenarios, 3600 steps (the gradient's workload): every gene of every printable
  genome against FP64 central differences (GPU, pe_objective), as test_gpu_grad.py checks 64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def generation(cuda, pe):
    torch = cuda
    pop, S = 100000, 12
    G = pe.random_genomes(2, pop)
    seeds = list(range(25, 25 + S))
    eng = pe.Engine(0)
    d_g = torch.from_numpy(G).cuda()
    dist = torch.empty(pop * S, device="cuda")
    steps = torch.empty(pop * S, dtype=torch.int32, device="cuda")
    scores = torch.empty(pop, device="cuda")
    eng.eval_batch(d_g, pop, seeds, 0, 7200, dist, steps, scores)
    torch.cuda.synchronize()
    out = dict(G=G, seeds=seeds, dist=dist.cpu().numpy().reshape(pop, S), steps=steps.cpu().numpy().reshape(pop, S),
               scores=scores.cpu().numpy(), eng=eng)
    yield out
    eng.close()


def test_full_generation_sample_matches_oracle(generation, oracle):
    from scipy.stats import spearmanr

    G, seeds = generation["G"], generation["seeds"]
    rng = np.random.default_rng(7)
    idx = np.sort(rng.choice(len(G), 300, replace=False))
    ref, ref_steps = oracle.eval_batch(G[idx], seeds, vary=0, max_steps=7200)
    ref = ref.reshape(len(idx), -1)
    got = generation["dist"][idx]
    np.testing.assert_array_equal(got == -100.0, ref == -100.0)
    np.testing.assert_array_equal(generation["steps"][idx] == 0, ref_steps.reshape(len(idx), -1) == 0)
    bad = np.abs(got - ref) > np.maximum(0.005 * np.abs(ref), 0.02)
    assert not bad.any(), (int(bad.sum()), float(np.abs(got - ref).max()))
    rs = oracle.robust_scores(ref.reshape(-1), len(idx), len(seeds))
    assert spearmanr(generation["scores"][idx], rs).statistic >= 0.999


def test_full_generation_permutation_invariant(generation, cuda):
    torch = cuda
    G, seeds, eng = generation["G"], generation["seeds"], generation["eng"]
    pop, S = G.shape[0], len(seeds)
    perm = np.random.default_rng(11).permutation(pop)
    d_g = torch.from_numpy(np.ascontiguousarray(G[perm])).cuda()
    dist = torch.empty(pop * S, device="cuda")
    eng.eval_batch(d_g, pop, seeds, 0, 7200, dist)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dist.cpu().numpy().reshape(pop, S), generation["dist"][perm])


def test_full_generation_scores_are_the_reduction_of_distances(generation, oracle):
    G, seeds = generation["G"], generation["seeds"]
    host = oracle.robust_scores(generation["dist"].reshape(-1), len(G), len(seeds))
    np.testing.assert_array_equal(generation["scores"], host)


def test_gradient_every_gene_of_full_c4(cuda, pe, engine, oracle):
    """Every gene of every printable genome of the gradient workload against FP64 central
    differences (GPU, pe_objective), with the population bar of gpu_helpers.check_grad_population."""
    from gpu_helpers import check_grad_population, fd64_per_gene

    torch = cuda
    pop, S = 256, 8
    G = pe.random_genomes(4, pop)
    seeds = list(range(1, S + 1))
    lo, hi = oracle.genome_bounds()
    d_g = torch.from_numpy(G).cuda()
    grad = torch.empty(pop, 35, device="cuda")
    obj = torch.empty(pop, device="cuda")
    engine.grad(d_g, pop, seeds, grad, max_steps=3600, d_obj=obj)
    torch.cuda.synchronize()
    grad = grad.cpu().numpy().astype(np.float64)
    live = np.flatnonzero(obj.cpu().numpy() > -100)
    fd, levels = fd64_per_gene(torch, engine, G[live], seeds, 3600, lo, hi)
    print("genes decided by step pairs 1e-4, 2e-5, 4e-6, 1e-6, 3e-7 of the range, none:", levels.tolist())
    check_grad_population(grad[live], fd, "C4, every printable genome:")
