"""pe_eval_batch_noalloc through the C ABI against pe_eval_batch.

The allocation-free entry point serves callers that cannot allocate device memory when they
evaluate (for example a host that reserves all device memory for its own pool, or a real-time
loop that must not enter the driver's allocator).  It must return what the allocating engine returns for the same
inputs; the two use the same body-frame formulation and every execution shape of it is
bit-identical, so the comparison is exact.  Two different calls run back to back, because the
static working memory keeps the previous call's contents.  This file is collected last.
"""
import numpy as np
import pytest

from gpu_helpers import dev

pytestmark = pytest.mark.gpu


def _engine_result(torch, pe, G, seeds, vary, max_steps=7200):
    eng = pe.Engine(0)  # default formulation and shape
    pop, S = G.shape[0], len(seeds)
    d = torch.empty(pop * S, device="cuda")
    st = torch.empty(pop * S, dtype=torch.int32, device="cuda")
    sc = torch.empty(pop, device="cuda")
    eng.eval_batch(dev(torch, G), pop, seeds, vary, max_steps, d, st, sc)
    torch.cuda.synchronize()
    eng.close()
    return d.cpu().numpy(), st.cpu().numpy(), sc.cpu().numpy()


def test_noalloc_matches_engine_on_two_calls_in_a_row(cuda, pe, oracle):
    torch = cuda
    # the last two cases: vary 1 with a short horizon (the engine flies it in one launch too),
    # and exactly the limits, 256 genomes x 16 scenarios = 4096 flights
    cases = [(oracle.grand(501, 200), [25 + s for s in range(12)], 0, 7200),
             (oracle.grand(502, 96), [9001 + 7919 * s for s in range(40)], 0, 7200),
             (oracle.grand(505, 128), [100003 + 7919 * s for s in range(8)], 1, 900),
             (oracle.grand(506, 256), [41 + s for s in range(16)], 0, 7200)]
    for G, seeds, vary, max_steps in cases:
        pop, S = G.shape[0], len(seeds)
        d = torch.full((pop * S,), 12345.0, device="cuda")
        st = torch.full((pop * S,), -7, dtype=torch.int32, device="cuda")
        sc = torch.full((pop,), 12345.0, device="cuda")
        pe.eval_batch_noalloc(dev(torch, G), pop, seeds, vary, max_steps, d, st, sc)
        torch.cuda.synchronize()
        want_d, want_st, want_sc = _engine_result(torch, pe, G, seeds, vary, max_steps)
        assert np.array_equal(d.cpu().numpy().view(np.uint32), want_d.view(np.uint32))
        assert np.array_equal(st.cpu().numpy(), want_st)
        assert np.array_equal(sc.cpu().numpy().view(np.uint32), want_sc.view(np.uint32))


def test_noalloc_scores_without_distance_buffer(cuda, pe, oracle):
    torch = cuda
    G = oracle.grand(503, 64)
    seeds = [3, 4, 5, 6]
    sc = torch.empty(64, device="cuda")
    pe.eval_batch_noalloc(dev(torch, G), 64, seeds, 0, 7200, None, None, sc)
    torch.cuda.synchronize()
    _, _, want = _engine_result(torch, pe, G, seeds, 0)
    assert np.array_equal(sc.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_memory(cuda, pe, oracle):
    torch = cuda
    G = dev(torch, oracle.grand(504, 300))
    with pytest.raises(pe.PEError) as e:
        pe.eval_batch_noalloc(G, 257, [1])
    assert e.value.code == pe.PE_EINVAL and "static working memory" in str(e.value)
    with pytest.raises(pe.PEError):
        pe.eval_batch_noalloc(G, 200, list(range(21)))  # 4200 flights
