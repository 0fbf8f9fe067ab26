"""The reference's drivers on the engine: evaluate (telemetry CSV + audit), select-best, evolve, and
the `planes` command line (src/sim.cu:258-520, src/main.cu:36-106)."""
import csv
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "planes-rl_gb300", "bin", "planes")


def _f32(x):
    return np.float32(x)


def test_evaluate_design_csv_and_audit(cuda, pe, engine, host_golden, tmp_path):
    genome = host_golden["presets"][0].astype(np.float32)
    csv_path = str(tmp_path / "sub" / "robust.csv")
    stats = np.zeros(18, np.float32)
    pe.LIB.pe_evaluate_design.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_void_p]
    assert pe.LIB.pe_evaluate_design(genome.ctypes.data, 64, 9001, csv_path.encode(), stats.ctypes.data) == 0
    rows = list(csv.reader(open(csv_path)))
    assert rows[0][:3] == ["scenario", "seed", "distance_m"] and len(rows[0]) == 28 and len(rows) == 65
    seeds = [9001 + 7919 * i for i in range(64)]
    assert [int(r[1]) for r in rows[1:]] == seeds
    want = engine.evaluate_population(genome[None], seeds)["dist"]
    got = np.array([float(r[2]) for r in rows[1:]], np.float32)
    assert np.allclose(got, want, atol=1e-6)  # %.6f in the CSV
    srt = np.sort(want)
    mean = _f32(0)
    for x in srt:
        mean = _f32(mean + _f32(x / _f32(64)))
    assert stats[5] == mean and stats[0] == srt[0] and stats[10] == srt[-1] and stats[17] == 64
    assert 0.005 < stats[13] < 0.1  # PLA mass in kg


def test_select_finalist_picks_best_robust_score(cuda, pe, engine, oracle, tmp_path):
    cands = oracle.grand(77, 6).astype(np.float32)
    out = str(tmp_path / "run")
    best = C.c_int(-1)
    pe.LIB.pe_select_finalist.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_void_p]
    assert pe.LIB.pe_select_finalist(cands.ctypes.data, 6, 128, 1900001, out.encode(), C.byref(best)) == 0
    seeds = [1900001 + 7919 * i for i in range(128)]
    dist = engine.evaluate_population(cands, seeds)["dist"]
    scores = oracle.robust_scores(dist, 6, 128)
    assert best.value == int(np.argmax(scores))
    rows = list(csv.reader(open(os.path.join(out, "finalist-selection.csv"))))
    assert rows[0] == ["candidate", "robust_score", "mean", "cvar25", "worst"] and len(rows) == 7
    assert np.allclose([float(r[1]) for r in rows[1:]], scores, atol=1e-5)
    assert np.array_equal(pe.load_best(os.path.join(out, "best-final.bin")), cands[best.value])


def test_run_ga_outputs_and_determinism(cuda, pe, tmp_path):
    outs = []
    for k in range(2):
        out = str(tmp_path / ("ga%d" % k))
        pe.LIB.pe_run_ga.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_char_p]
        assert pe.LIB.pe_run_ga(128, 3, 2, out.encode(), None) == 0
        hist = list(csv.reader(open(os.path.join(out, "history.csv"))))
        assert hist[0] == ["gen", "train_best", "holdout128", "mean", "p90"] and len(hist) == 4
        pop = pe.load_genomes(os.path.join(out, "pop.bin"))
        arch = pe.load_genomes(os.path.join(out, "archive.bin"))
        assert pop.shape == (128, 35) and arch.shape == (3, 35)
        lo, hi = pe.genome_bounds()
        assert np.all(pop >= lo) and np.all(pop <= hi)
        outs.append([open(os.path.join(out, f), "rb").read() for f in ("history.csv", "pop.bin", "best.bin")])
    assert outs[0] == outs[1]


def test_cli_evaluate_and_errors(cuda, pe, host_golden, tmp_path):
    best = str(tmp_path / "best.bin")
    pe.save_best(best, host_golden["presets"][1])
    csv_path = str(tmp_path / "r.csv")
    r = subprocess.run([CLI, "evaluate", "--best", best, "--n", "16", "--seed", "9001", "--o", csv_path],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "robustness audit: 16 GPU scenarios" in r.stdout and os.path.exists(csv_path)
    r = subprocess.run([CLI, "showcase"], capture_output=True, text=True)
    assert r.returncode == 1 and "renderer" in r.stderr
    r = subprocess.run([CLI, "evaluate", "--best", str(tmp_path / "missing.bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "missing" in r.stderr


def test_cli_evolve_on_device(cuda, pe, tmp_path):
    """planes evolve --device 1: the device GA with Adam polish, writing best.bin and history.csv."""
    out = str(tmp_path / "dev")
    r = subprocess.run([CLI, "evolve", "--device", "1", "--pop", "128", "--gens", "3", "--seeds", "2", "--seed", "5",
                        "--polish-top", "8", "--polish-steps", "1", "--audit", "32", "--out", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "best holdout score" in r.stdout and "3 gradient calls" in r.stdout and "audit on 32 scenarios" in r.stdout
    rows = open(os.path.join(out, "history.csv")).read().strip().splitlines()
    assert rows[0] == "gen,train_best,holdout128,mean,p90,gpu_s" and len(rows) == 4
    assert os.path.getsize(os.path.join(out, "best.bin")) == 35 * 4
    r = subprocess.run([CLI, "evolve", "--device", "1", "--init", "x.bin", "--out", out], capture_output=True, text=True)
    assert r.returncode == 1 and "host GA" in r.stderr


def test_run_ga_error_paths_close_history_once(cuda, pe, tmp_path):
    """An evaluation that fails inside run_ga (injected on the host: the training batch of generation 0,
    then the holdout batch) returns its status with history.csv closed exactly once; the next run
    succeeds."""
    pe.LIB.pe_run_ga.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_char_p]
    try:
        for after, name in ((0, "train"), (1, "holdout")):
            out = str(tmp_path / name)
            assert pe.LIB.pe_debug_fail_evaluations(after) == pe.PE_OK
            assert pe.LIB.pe_run_ga(64, 2, 2, out.encode(), None) == pe.PE_ECUDA
            assert b"injected evaluation failure" in pe.LIB.pe_last_error()
            assert open(os.path.join(out, "history.csv")).read() == "gen,train_best,holdout128,mean,p90\n"
    finally:
        pe.LIB.pe_debug_fail_evaluations(-1)
    out = str(tmp_path / "ok")
    assert pe.LIB.pe_run_ga(64, 2, 2, out.encode(), None) == 0
    assert len(open(os.path.join(out, "history.csv")).read().strip().splitlines()) == 3
