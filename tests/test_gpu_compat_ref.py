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


C3 = os.path.join(os.path.dirname(GOLDEN), "ref_cuda_c3_slice.npz")
TRAJ = os.path.join(os.path.dirname(GOLDEN), "ref_cuda_traj.npz")


@pytest.mark.skipif(not os.path.exists(C3), reason="reference CUDA slice of the 100k x 12 generation not recorded")
def test_c3_slice_matches_reference_cuda_build(cuda, any_engine, oracle):
    """The first 10,000 genomes of the 100,000 x 12 generation (std::mt19937(2), env seeds 25..36,
    vary 0) against the reference build's own fitness: at least 99 % of flights within 0.5 % (or
    5 mm below 1 m), oversize exact, Spearman of the tail-aware scores >= 0.999."""
    torch = cuda
    engine = any_engine
    gold = np.load(C3)
    ref = gold["fitness"]
    pop, S = ref.shape
    G = oracle.grand(int(gold["genome_seed"]), pop)
    out = eval_gpu(torch, engine, G, [int(x) for x in gold["seeds"]])
    ref = ref.reshape(-1)
    assert np.array_equal(out["dist"] == -100, ref == -100)
    within = np.mean(np.abs(out["dist"] - ref) <= 0.005 * np.maximum(np.abs(ref), 1.0))
    printable = ref > -100
    same = np.mean(out["dist"][printable].view(np.uint32) == ref[printable].view(np.uint32))
    rho = spearman(out["scores"], oracle.robust_scores(ref, pop, S))
    print("formulation %d, %d x %d vs reference CUDA build: within 0.5%% %.5f, bit-identical (printable) %.4f, "
          "spearman %.10f, max |diff| %.4f m" % (engine.config.formulation, pop, S, within, same, rho,
                                                  np.abs(out["dist"] - ref).max()))
    assert within >= 0.99 and rho >= 0.999


def _state16(st15, k):
    """Reference PlaneState (pos q vel wb done fitness) at step k -> the C ABI's 16-float state, the
    clock restarted at k * SIM_DT as the reference's resumed launch does (src/sim.cu:108-112)."""
    s = np.zeros((st15.shape[0], 16), np.float32)
    s[:, :13] = st15[:, :13]
    s[:, 13] = np.float32(k) * (np.float32(1.0) / np.float32(600.0))
    s[:, 14] = np.full(st15.shape[0], k, np.int32).view(np.float32)
    return s


@pytest.mark.skipif(not os.path.exists(TRAJ), reason="reference CUDA trajectory states not recorded")
@pytest.mark.parametrize("formulation,lanes", [(0, 32), (1, 16), (1, 32)])
def test_teacher_forced_steps_match_reference_cuda_build(cuda, pe, oracle, formulation, lanes):
    """One step from the reference build's own states at steps 1, 7, 60, 599, 600 and 601 (64 genomes,
    vary 1), in both formulations, against the reference build's step from the same state.  A step's
    aerodynamic force F and torque tau reach the state only through v += dt F / m and
    w += dt I^-1 tau, so the 1e-5 force bar is checked on those increments at the resolution a float32
    state allows: |dv - dv_ref| <= 1e-5 dt max(|F|, m g) / m + 2 sqrt(3) ulp(v) and
    |dw - dw_ref| <= 1e-5 dt |I^-1| max(|tau|, chord m g) + 2 sqrt(3) ulp(w), with |F|, |tau|, the
    printed m and I^-1 from the FP64 oracle at that state -- the floors of the teacher-forced test
    against FP64.  Positions and attitudes within 1e-5 relative; the end-of-flight flags equal."""
    torch = cuda
    gold = np.load(TRAJ)
    engine = pe.Engine(0)
    engine.set_config(formulation=formulation, reg_cap=0, lanes=lanes)
    G = oracle.grand(int(gold["genome_seed"]), gold["state_in"].shape[1])
    seed, vary = int(gold["seed"]), int(gold["vary"])
    pop = len(G)
    pre64 = oracle.Prepared(G, 64)
    eval_gpu(torch, engine, G, [seed], vary=vary, max_steps=1, scores=False)
    dt = 1.0 / 600.0
    worst_v = worst_w = 0.0
    checked = 0
    for k, sin15, sout15 in zip(gold["steps"], gold["state_in"], gold["state_out"]):
        k = int(k)
        live = (sin15[:, 13] == 0) & np.all(np.isfinite(sin15[:, :13]), axis=1) & (pre64.nt > 0)
        sin16 = _state16(sin15, k)
        d_in = dev(torch, sin16)
        d_out = torch.empty_like(d_in)
        FT = torch.empty(pop, 6, device="cuda")
        done = torch.empty(pop, dtype=torch.int32, device="cuda")
        fit = torch.empty(pop, device="cuda")
        engine.debug_step(pop, [seed], vary, 7200, d_in, d_out, FT, done, fit, k, lanes=lanes)
        torch.cuda.synchronize()
        mine = d_out.cpu().numpy()
        assert np.array_equal(done.cpu().numpy()[live] != 0, sout15[live, 13] != 0), k
        for p in np.flatnonzero(live):
            env = seed + p * 7919
            a, b, x0 = mine[p], sout15[p], sin15[p]
            for sl in (slice(0, 3), slice(3, 7)):
                assert np.linalg.norm(a[sl] - b[sl]) <= 1e-5 * max(np.linalg.norm(b[sl]), 1e-3), (k, p, sl)
            st = np.zeros(16)
            st[:13] = x0[:13]
            st[13] = float(sin16[p, 13])
            _, ft = pre64.step(p, env, st, k)
            pmp, _ = oracle.printed_mass_props(pre64.mp[p], oracle.scenario_desc(env, 64), 64)
            m, inv_i = pmp[0], pmp[11:20].reshape(3, 3)
            floor_v = 1e-5 * dt * max(np.linalg.norm(ft[:3]), m * 9.81) / m
            floor_w = 1e-5 * dt * np.linalg.norm(inv_i, 2) * max(np.linalg.norm(ft[3:]), G[p, 1] * m * 9.81)
            for sl, floor, name in ((slice(7, 10), floor_v, "v"), (slice(10, 13), floor_w, "w")):
                rnd = 2 * np.sqrt(3) * float(np.spacing(np.abs(b[sl]).max()))
                err = float(np.linalg.norm(a[sl].astype(np.float64) - b[sl]))
                assert err <= floor + rnd, (k, p, name, err, floor, rnd)
                rel = max(err - rnd, 0.0) / floor * 1e-5  # the error in units of the force bar
                if name == "v":
                    worst_v = max(worst_v, rel)
                else:
                    worst_w = max(worst_w, rel)
            checked += 1
    engine.close()
    print("formulation %d, %d lanes: %d teacher-forced steps vs the reference build; force / torque error beyond "
          "state rounding, relative to max(|F|, m g) / max(|tau|, chord m g): %.2e / %.2e" %
          (formulation, lanes, checked, worst_v, worst_w))
    assert checked >= 120
