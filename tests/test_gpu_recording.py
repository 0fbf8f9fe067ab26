"""Pose recording and the showcase launch grid of the reference's gpu_sim (src/sim.cu:72-79,
115-128) through pe_sim, against the oracle's restatement of that loop (oracle fly_rec, FP32).

Positions are compared within the path's distance bar (2 cm + 0.5 %), attitudes within 0.02 rad
of rotation: the default body-frame kernel and the reference's arithmetic round differently,
and the difference grows over a tumbling flight.
Alive flags, record slots (including the reference's slot restart at every 600-step launch)
and the frozen pose after landing are compared exactly.
"""
import numpy as np
import pytest

from gpu_helpers import dev

pytestmark = pytest.mark.gpu


def _sim_rec(cuda, pe, G, seed, rec_every, rec_cap, spread=0.0, vary=0):
    torch = cuda
    pop = len(G)
    pb = pe.PanelBuf(pop)
    pb.prepare(dev(torch, G), pop)
    fit = torch.empty(pop, device="cuda")
    rec = torch.full((pop, max(rec_cap, 1), 8), float("nan"), device="cuda")
    pb.sim(pop, seed, fit, d_rec=rec, rec_every=rec_every, rec_cap=rec_cap, spread=spread, vary=vary)
    fit_plain = torch.empty(pop, device="cuda")
    if spread == 0.0:
        pb.sim(pop, seed, fit_plain, vary=vary)
    pb.free()
    torch.cuda.synchronize()
    return fit.cpu().numpy(), rec.cpu().numpy()[:, :rec_cap], fit_plain.cpu().numpy()


def _check_against_oracle(oracle, G, fit, rec, seed, rec_every, rec_cap, spread=0.0, vary=0):
    pre = oracle.Prepared(G, prec=32)
    for p in range(len(G)):
        env = seed + (p * 7919 if vary else 0)
        want, wfit = pre.fly_rec(p, env, spread, rec_every, rec_cap)
        got = rec[p]
        # unwritten slots (NaN on both sides: the buffer's fill and the oracle's) must agree too
        np.testing.assert_array_equal(got[:, 7], want[:, 7], err_msg="alive flags of plane %d" % p)
        w = ~np.isnan(want[:, 7])
        got, want = got[w], want[w]
        dpos = np.abs(got[:, :3] - want[:, :3])
        assert (dpos <= 0.02 + 0.005 * np.abs(want[:, :3])).all(), (p, dpos.max())
        ang = 2 * np.arccos(np.clip(np.abs((got[:, 3:7].astype(np.float64) * want[:, 3:7]).sum(axis=1)), 0, 1))
        assert ang.max() <= 0.02, (p, ang.max())
        if wfit == -100.0:
            assert fit[p] == -100.0
        else:
            assert abs(fit[p] - wfit) <= 0.02 + 0.005 * abs(wfit), (p, fit[p], wfit)
        alive = got[:, 7] == 1
        frozen = got[~alive]
        if pre.nt[p] > 0 and len(frozen):  # after landing every frame is the final pose
            assert (frozen == frozen[-1]).all()
            if wfit > -10 and frozen[-1][2] <= 0.0:
                assert frozen[-1][0] == fit[p]  # landed: the fitness is the final x


def test_recording_every_10_matches_reference_loop(cuda, pe, oracle):
    G = oracle.grand(11, 48)
    fit, rec, plain = _sim_rec(cuda, pe, G, 25, 10, 720)
    np.testing.assert_array_equal(fit, plain)  # recording does not change the flights
    _check_against_oracle(oracle, G, fit, rec, 25, 10, 720)


def test_recording_slot_restart_and_cap(cuda, pe, oracle):
    """rec_every = 7 does not divide 600: each launch restarts at step0 / 7 and overwrites the
    previous launch's last slot, as the reference does; rec_cap cuts the record short."""
    G = oracle.grand(12, 24)
    fit, rec, plain = _sim_rec(cuda, pe, G, 31, 7, 1100)
    np.testing.assert_array_equal(fit, plain)
    _check_against_oracle(oracle, G, fit, rec, 31, 7, 1100)
    fit4, rec4, _ = _sim_rec(cuda, pe, G, 31, 7, 4)
    np.testing.assert_array_equal(rec4, rec[:, :4])


def test_launch_grid_and_vary(cuda, pe, oracle):
    G = oracle.grand(13, 60)  # planes 0..59 span three rows of the 25-column grid
    fit, rec, _ = _sim_rec(cuda, pe, G, 5, 20, 360, spread=0.5, vary=1)
    _check_against_oracle(oracle, G, fit, rec, 5, 20, 360, spread=0.5, vary=1)
    p = np.arange(len(G))
    np.testing.assert_array_equal(rec[:, 0, 0], (-(p // 25) * np.float32(0.5) * np.float32(1.4)).astype(np.float32))
    np.testing.assert_array_equal(rec[:, 0, 1], ((p % 25 - 12) * np.float32(0.5)).astype(np.float32))


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)),
                                    "golden", "ref_cuda_golden.npz")


def test_recording_matches_reference_cuda_build(cuda, pe):
    """Against the reference's own CUDA build (its k_sim driven by gpu_sim with d_rec and the launch
    grid, tests/golden/make_ref_cuda_golden.py): every slot, alive flag and unwritten slot exactly,
    poses within the distance bar and 0.02 rad, fitness within the distance bar, oversize exactly."""
    gold = np.load(GOLDEN)
    if "rec" not in gold.files:
        pytest.skip("reference recording not in the golden vectors")
    G = gold["rec_genomes"]
    seed, vary, every, cap = (int(x) for x in gold["rec_params"])
    fit, rec, _ = _sim_rec(cuda, pe, G, seed, every, cap, spread=float(gold["rec_spread"]), vary=vary)
    want, wfit = gold["rec"], gold["rec_fitness"]
    np.testing.assert_array_equal(rec[..., 7], want[..., 7])  # alive flags (NaN where unwritten)
    w = ~np.isnan(want[..., 7])
    got, ref = rec[w], want[w]
    dpos = np.abs(got[:, :3] - ref[:, :3])
    assert (dpos <= 0.02 + 0.005 * np.abs(ref[:, :3])).all(), float(dpos.max())
    ang = 2 * np.arccos(np.clip(np.abs((got[:, 3:7].astype(np.float64) * ref[:, 3:7]).sum(axis=1)), 0, 1))
    assert ang.max() <= 0.02, float(ang.max())
    np.testing.assert_array_equal(fit == -100.0, wfit == -100.0)
    ok = wfit != -100.0
    assert (np.abs(fit[ok] - wfit[ok]) <= 0.02 + 0.005 * np.abs(wfit[ok])).all()
    # the launch grid's first frame is the reference's own offsets
    np.testing.assert_array_equal(rec[:, 0, :2], want[:, 0, :2])
