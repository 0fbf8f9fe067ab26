"""The robustness audit on the device (pe_distance_stats, pe_audit; src/sim.cu:291-309 with the
percentile of src/sim.cu:250-256) against the oracle's statistics (or_audit_stats): bit for bit.

Sizes cover one key, the 1024-key block of the sort and its neighbours, non-powers of two and a
100,000-scenario audit (the reference's `make evaluate` size)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 3, 1000, 1024, 1025, 4097, 100003])
def test_distance_stats_bit_exact(cuda, pe, oracle, n):
    torch = cuda
    rng = np.random.default_rng(n)
    d = rng.normal(6.0, 4.0, n).astype(np.float32)
    d[rng.integers(0, n, max(1, n // 7))] = -100.0  # oversize rows
    d[rng.integers(0, n, max(1, n // 5))] = 3.25  # ties
    st = torch.empty(pe.AUDIT_STATS, device="cuda")
    pe.distance_stats(torch.from_numpy(d).cuda(), n, st)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(st.cpu().numpy().view(np.uint32), oracle.audit_stats(d).view(np.uint32))


def test_distance_stats_rejects_bad_sizes(cuda, pe):
    torch = cuda
    d = torch.zeros(4, device="cuda")
    st = torch.empty(pe.AUDIT_STATS, device="cuda")
    for n in (0, -1, (1 << 26) + 1):
        with pytest.raises(pe.PEError):
            pe.distance_stats(d, n, st)
    with pytest.raises(pe.PEError):
        pe.distance_stats(None, 4, st)


def test_audit_100k_scenarios(cuda, pe, engine, oracle, host_golden):
    genome = host_golden["presets"][0].astype(np.float32)
    seeds = [9001 + 7919 * i for i in range(100000)]
    out = engine.audit(genome, seeds, want_dist=True)
    np.testing.assert_array_equal(out["stats"].view(np.uint32), oracle.audit_stats(out["dist"]).view(np.uint32))
    want = engine.evaluate_population(genome[None], seeds, want_steps=False, want_scores=False)["dist"]
    np.testing.assert_array_equal(out["dist"], want)
    t0 = time.perf_counter()
    out2 = engine.audit(genome, seeds)  # statistics only: no distances cross to the host
    dt = time.perf_counter() - t0
    np.testing.assert_array_equal(out2["stats"], out["stats"])
    print("audit of 100,000 scenarios on the device: %.1f ms; %s" %
          (dt * 1e3, dict(zip(pe.AUDIT_NAMES, np.round(out["stats"], 3).tolist()))))
