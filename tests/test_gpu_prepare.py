"""GPU mesh / mass properties / panels against the oracle (and the reference CUDA build)."""
import os

import numpy as np
import pytest

from gpu_helpers import eval_gpu, plane_table

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _genomes(oracle, host_golden):
    return np.concatenate([host_golden["genomes"], oracle.grand(11, 400)]).astype(np.float32)


def test_plane_table_matches_oracle(cuda, engine, oracle, host_golden):
    torch = cuda
    G = _genomes(oracle, host_golden)
    pop = G.shape[0]
    eval_gpu(torch, engine, G, [1], max_steps=1, scores=False)
    t = plane_table(torch, engine, pop)
    ref = oracle.Prepared(G)
    # printability and triangle counts: exact
    assert np.array_equal(t["nt"], ref.nt)
    assert np.array_equal(t["ext"][:, 3].astype(np.int32)[ref.nt > 0], ref.nt[ref.nt > 0])
    # exact per-plane prefix ranges of the topology triangle counts
    topo = t["ext"][:, 3].astype(np.int64)
    assert np.array_equal(t["off"], np.concatenate([[0], np.cumsum(topo)[:-1]]))
    # mass properties (fast-math sin/cos/tan/sqrt in the mesher vs host libm)
    mp, rmp = t["mp"], ref.mp
    assert np.all(np.abs(mp[:, 0] - rmp[:, 0]) <= 1e-5 * rmp[:, 0])
    chord = G[:, 1][:, None]
    assert np.all(np.abs(mp[:, 2:5] - rmp[:, 2:5]) <= 2e-6 * chord)
    iscale = rmp[:, 5:8].max(1, keepdims=True)
    assert np.all(np.abs(mp[:, 5:11] - rmp[:, 5:11]) <= 2e-5 * iscale)
    # the 3x3 inverse (FP64 on the GPU) against the FP64 oracle
    r64 = oracle.Prepared(G[:64], prec=64)
    inv, rinv = mp[:64, 11:], r64.mp[:, 11:]
    iv_scale = np.abs(rinv).max(1, keepdims=True)
    assert np.all(np.abs(inv - rinv) <= 1e-4 * iv_scale)
    # panels, packed at the plane offsets
    for p in range(pop):
        n = int(ref.nt[p])
        if n == 0:
            continue
        o = int(t["off"][p])
        pc, pn = t["pc"][o:o + n], t["pn"][o:o + n]
        scale = float(G[p, 1])
        assert np.all(np.abs(pc[:, :3] - ref.pc[p, :n, :3]) <= 2e-6 * scale), p
        assert np.all(np.abs(pc[:, 3] - ref.pc[p, :n, 3]) <= 1e-4 * np.abs(ref.pc[p, :n, 3]) + 1e-12), p
        big = ref.pc[p, :n, 3] > 1e-6  # normals of sliver panels are ill-conditioned
        assert np.all(np.abs(pn[big, :3] - ref.pn[p, :n, :3][big]) <= 1e-4), p


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "ref_cuda_golden.npz")),
                    reason="reference CUDA golden vectors not recorded")
def test_plane_table_matches_reference_cuda_build(cuda, engine):
    """Against the reference build's own k_prepare output: triangle counts exact, mass
    properties and panels to FP32 rounding (the bit-identical share is reported)."""
    torch = cuda
    gold = np.load(os.path.join(GOLDEN, "ref_cuda_golden.npz"))
    G = gold["c1_genomes"]
    pop = G.shape[0]
    eval_gpu(torch, engine, G, [1], max_steps=1, scores=False)
    t = plane_table(torch, engine, pop)
    assert np.array_equal(t["nt"], gold["c1_nt"])
    mp, rmp = t["mp"], gold["c1_mp"]
    same = np.mean(np.all(mp[:, :11].view(np.uint32) == rmp[:, :11].view(np.uint32), 1))
    print("mass properties bit-identical to the reference build: %.3f of planes" % same)
    assert np.all(np.abs(mp[:, 0] - rmp[:, 0]) <= 1e-6 * rmp[:, 0])
    assert np.all(np.abs(mp[:, 2:5] - rmp[:, 2:5]) <= 1e-6 * G[:, 1:2])
    iscale = rmp[:, 5:8].max(1, keepdims=True)
    assert np.all(np.abs(mp[:, 5:11] - rmp[:, 5:11]) <= 1e-5 * iscale)
    for p in range(gold["c1_pc"].shape[0]):
        n = int(gold["c1_nt"][p])
        o = int(t["off"][p])
        ref_pc, ref_pn = gold["c1_pc"][p, :n], gold["c1_pn"][p, :n]
        assert np.all(np.abs(t["pc"][o:o + n, :3] - ref_pc[:, :3]) <= 1e-6 * G[p, 1]), p
        assert np.all(np.abs(t["pc"][o:o + n, 3] - ref_pc[:, 3]) <= 1e-5 * ref_pc[:, 3] + 1e-12), p
        big = ref_pc[:, 3] > 1e-6
        assert np.all(np.abs(t["pn"][o:o + n, :3][big] - ref_pn[big, :3]) <= 1e-5), p


def test_prefix_ranges_beyond_a_million_planes(cuda, pe):
    """1,048,577 planes: the block totals of the prefix scan span two tiles of 1,024 blocks, so the
    offsets of the planes past 2^20 carry the first tile's sum.  Checked against a host prefix sum of
    the topology triangle counts; the last planes fly their first step bit-identically to the same
    genomes in a batch of their own (overlapping panel ranges would change their forces)."""
    torch = cuda
    pop = (1 << 20) + 1
    G = pe.random_genomes(31, pop)
    eng = pe.Engine(0)
    try:
        big = eval_gpu(torch, eng, G, [5], max_steps=2, scores=False)
        nt = torch.empty(pop, dtype=torch.int32, device="cuda")
        off = torch.empty(pop, dtype=torch.int32, device="cuda")
        ext = torch.empty(pop, 4, dtype=torch.float32, device="cuda")
        total = eng.plane_table(pop, d_nt=nt, d_off=off, d_ext=ext)
        torch.cuda.synchronize()
        topo = ext[:, 3].cpu().numpy().astype(np.int64)
        want = np.concatenate([[0], np.cumsum(topo)[:-1]])
        assert np.array_equal(off.cpu().numpy().astype(np.int64), want)
        assert total == int(topo.sum())
        ntv = nt.cpu().numpy()
        assert np.all((ntv == 0) | (ntv == topo))
        tail = 3000
        alone = eval_gpu(torch, eng, G[-tail:], [5], max_steps=2, scores=False)
        assert np.array_equal(big["dist"][-tail:].view(np.uint32), alone["dist"].view(np.uint32))
        assert np.array_equal(big["steps"][-tail:], alone["steps"])
        assert (big["steps"][-tail:] > 0).mean() > 0.5
        with pytest.raises(pe.PEError) as e:
            eng.eval_batch(torch.empty(1, 35, device="cuda"), pe.MAX_POP + 1, [1], max_steps=1)
        assert e.value.code == pe.PE_EINVAL
    finally:
        eng.close()
