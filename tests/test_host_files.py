"""The evolve/evaluate file formats on the host (no GPU): best.bin is one raw 140-byte genome
(src/sim.cu:327-331); pop.bin / archive.bin are int32 n + n genomes (src/sim.cu:333-338,
src/main.cu:28-34).  Corrupt inputs are errors, never crashes."""
import os

import numpy as np
import pytest


def test_genome_files_round_trip(built_lib, tmp_path):
    import pe

    G = pe.random_genomes(3, 10)
    p = str(tmp_path / "pop.bin")
    pe.save_genomes(p, G)
    assert os.path.getsize(p) == 4 + 10 * 140
    assert np.frombuffer(open(p, "rb").read(4), np.int32)[0] == 10
    np.testing.assert_array_equal(pe.load_genomes(p), G)
    np.testing.assert_array_equal(pe.load_genomes(p, cap=4), G[:4])
    b = str(tmp_path / "best.bin")
    pe.save_best(b, G[7])
    assert os.path.getsize(b) == 140
    np.testing.assert_array_equal(pe.load_best(b), G[7])


def test_corrupt_and_missing_files_are_errors(built_lib, tmp_path):
    import pe

    G = pe.random_genomes(4, 10)
    p = str(tmp_path / "pop.bin")
    pe.save_genomes(p, G)
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-70])  # the header says 10 genomes, 9.5 follow
    with pytest.raises(pe.PEError) as e:
        pe.load_genomes(p)
    assert e.value.code == pe.PE_EINVAL and "truncated" in str(e.value)
    open(p, "wb").write(b"\x01\x00")  # not even a count
    with pytest.raises(pe.PEError) as e:
        pe.load_genomes(p)
    assert "count" in str(e.value)
    with pytest.raises(pe.PEError):
        pe.load_genomes(str(tmp_path / "missing.bin"))
    b = str(tmp_path / "best.bin")
    open(b, "wb").write(b"\x00" * 100)
    with pytest.raises(pe.PEError) as e:
        pe.load_best(b)
    assert "140 bytes" in str(e.value)


def test_warm_start_is_clamped_to_the_bounds(built_lib):
    import pe

    lo, hi = pe.genome_bounds()
    g = np.stack([lo - 1.0, hi + 1.0, (lo + hi) / 2]).astype(np.float32)
    out = pe.sanitize_genomes(g.copy())
    np.testing.assert_array_equal(out[0], lo)
    np.testing.assert_array_equal(out[1], hi)
    np.testing.assert_array_equal(out[2], g[2])
