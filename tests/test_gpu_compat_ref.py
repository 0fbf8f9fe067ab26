"""The reference-compatible boundary (panelbuf_alloc / gpu_prepare / gpu_sim) and parity with the
reference's own CUDA build (golden vectors recorded by tests/golden/make_ref_cuda_golden.py)."""
import os

import numpy as np
import pytest

from gpu_helpers import dev, eval_gpu, spearman

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cuda_golden.npz")
need_golden = pytest.mark.skipif(not os.path.exists(GOLDEN), reason="reference CUDA golden vectors not recorded")


def test_panelbuf_path_equals_batched_engine(cuda, pe, engine, oracle):
    torch = cuda
    G = oracle.grand(9, 150)
    pop = len(G)
    g = dev(torch, G)
    pb = pe.PanelBuf(pop)
    pb.prepare(g, pop)
    fit = torch.empty(pop, device="cuda")
    for seed, vary in ((17, 0), (9001, 1)):
        pb.sim(pop, seed, fit, vary=vary)
        got = fit.cpu().numpy()
        want = eval_gpu(torch, engine, G, [seed], vary=vary, scores=False)["dist"]
        assert np.array_equal(got, want)
    with pytest.raises(pe.PEError) as e:
        pb.sim(pop, 1, fit, d_rec=fit, rec_every=0, rec_cap=4)
    assert e.value.code == pe.PE_EINVAL
    with pytest.raises(pe.PEError):
        pb.sim(pop + 1, 1, fit)
    pb.free()


@need_golden
def test_fitness_matches_reference_cuda_build(cuda, any_engine):
    """C1-style population (512 genomes x the GA's 8 seeds of generation 0, vary 0)."""
    torch = cuda
    engine = any_engine
    gold = np.load(GOLDEN)
    G, seeds = gold["c1_genomes"], gold["c1_seeds"]
    out = eval_gpu(torch, engine, G, list(seeds))
    ref = gold["c1_fitness"].reshape(-1)
    same = np.mean(out["dist"].view(np.uint32) == ref.view(np.uint32))
    within = np.mean(np.abs(out["dist"] - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0))
    from oracle_py import robust_scores
    rho = spearman(out["scores"], robust_scores(ref, len(G), len(seeds)))
    print("formulation %d vs reference CUDA build: bit-identical %.4f, within 0.5%% %.4f, spearman %.6f" %
          (engine.config.formulation, same, within, rho))
    assert within >= 0.99 and rho >= 0.999


@need_golden
def test_evaluate_style_vary_matches_reference_cuda_build(cuda, any_engine):
    torch = cuda
    engine = any_engine
    gold = np.load(GOLDEN)
    out = eval_gpu(torch, engine, gold["ev_genomes"], [int(gold["ev_seed"])], vary=1, scores=False)
    ref = gold["ev_fitness"]
    within = np.mean(np.abs(out["dist"] - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0))
    assert within >= 0.95


@need_golden
def test_release_and_step_match_reference_cuda_build(cuda, pe):
    """Release states and one resumed step in the reference arithmetic against the reference build."""
    torch = cuda
    engine = pe.Engine(0)
    engine.set_config(formulation=0, reg_cap=0, lanes=32)
    gold = np.load(GOLDEN)
    G, seed = gold["st_genomes"], int(gold["st_seed"])
    pop = len(G)
    eval_gpu(torch, engine, G, [seed], vary=1, max_steps=1, scores=False)
    st = torch.empty(pop, 16, device="cuda")
    engine.debug_release(pop, [seed], 1, st)
    torch.cuda.synchronize()
    mine = st.cpu().numpy()
    rel = gold["rel_states"]
    live = rel[:, 13] == 0  # PlaneState.done
    same = np.mean(np.all(mine[live, :13].view(np.uint32) == rel[live, :13].view(np.uint32), 1))
    for sl in (slice(0, 3), slice(3, 7), slice(7, 10), slice(10, 13)):
        a, b = mine[live, sl], rel[live, sl]
        assert np.all(np.linalg.norm(a - b, axis=1) <= 1e-5 * np.maximum(np.linalg.norm(b, axis=1), 1e-3)), sl
    # one resumed step from the reference's release states (clock = 1 * dt, step index 1)
    sin = np.zeros((pop, 16), np.float32)
    sin[:, :13] = rel[:, :13]
    sin[:, 13] = np.float32(1) * (np.float32(1.0) / np.float32(600.0))
    sin[:, 14] = np.array([1] * pop, np.int32).view(np.float32)
    d_in = dev(torch, sin)
    d_out = torch.empty_like(d_in)
    FT = torch.empty(pop, 6, device="cuda")
    done = torch.empty(pop, dtype=torch.int32, device="cuda")
    fit = torch.empty(pop, device="cuda")
    engine.debug_step(pop, [seed], 1, 7200, d_in, d_out, FT, done, fit, 1)
    torch.cuda.synchronize()
    nxt = d_out.cpu().numpy()
    ref = gold["st_out"]
    same_step = np.mean(np.all(nxt[live, :13].view(np.uint32) == ref[live, :13].view(np.uint32), 1))
    print("reference build: release bit-identical %.3f, one step bit-identical %.3f" % (same, same_step))
    for sl in (slice(0, 3), slice(3, 7), slice(7, 10), slice(10, 13)):
        a, b = nxt[live, sl], ref[live, sl]
        assert np.all(np.linalg.norm(a - b, axis=1) <= 1e-5 * np.maximum(np.linalg.norm(b, axis=1), 1e-3)), sl
    engine.close()
