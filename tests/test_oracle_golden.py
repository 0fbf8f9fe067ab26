"""The oracle against golden vectors recorded from the reference's own host code.

tests/golden/host_golden.npz comes from src/common.h + src/designs.cu of the reference,
compiled and run by tests/golden/make_host_golden.py.  Float results must match bit for bit.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_mesh_bit_exact(oracle, host_golden):
    g = host_golden
    for i, genome in enumerate(g["genomes"]):
        V, T = oracle.build_mesh(genome)
        nv, nt = int(g["nv"][i]), int(g["nt"][i])
        assert V.shape[0] == nv and T.shape[0] == nt, i
        assert np.array_equal(bits(V), bits(g["V"][i, :nv])), "vertices of genome %d" % i
        assert np.array_equal(T, g["T"][i, :nt]), "triangles of genome %d" % i


def test_printability_extent_mass_props_bit_exact(oracle, host_golden):
    g = host_golden
    for i, genome in enumerate(g["genomes"]):
        V, T = oracle.build_mesh(genome)
        assert int(oracle.fits_print_volume(V)) == int(g["printable"][i]), i
        assert np.array_equal(bits(oracle.mesh_extent(V)), bits(g["extent"][i])), i
        assert np.array_equal(bits(oracle.mass_props(genome, V, T)), bits(g["mp"][i])), i


def test_scenario_print_variation_gusts_bit_exact(oracle, host_golden):
    g = host_golden
    G = g["genomes"].shape[0]
    for k, seed in enumerate(g["scen_seeds"]):
        d = oracle.scenario_desc(int(seed))
        assert np.array_equal(bits(d), bits(g["scen"][k])), "scenario seed %d" % seed
        pm, cg = oracle.printed_mass_props(g["mp"][k % G], d)
        assert np.array_equal(bits(pm), bits(g["printed"][k])), "printed mass props seed %d" % seed
        assert np.array_equal(bits(cg), bits(g["cg"][k]))
        w = oracle.wind_at(g["wind_p"][k], float(g["wind_t"][k]), int(seed))
        assert np.array_equal(bits(w), bits(g["wind"][k])), "wind seed %d" % seed


def test_topology_counts(oracle, host_golden):
    """nt in {176,178,180} (mono) / {340,342,344} (biplane); nv <= 241 (bounds the device buffers)."""
    nts = set(int(x) for x in host_golden["nt"])
    assert nts <= {176, 178, 180, 340, 342, 344}
    assert int(host_golden["nv"].max()) <= 241
    for genome in oracle.grand(99, 400):
        V, T = oracle.build_mesh(genome)
        assert T.shape[0] in (176, 178, 180, 340, 342, 344) and V.shape[0] <= 241


def test_reference_geometry_invariants_on_presets(oracle, host_golden):
    """The assertions of the reference's tests/geometry_test.cpp:19-35, on its five presets."""
    for i, genome in enumerate(host_golden["presets"]):
        V, T = oracle.build_mesh(genome)
        # mirror symmetry of the wing grid (geometry_test.cpp:19-23): vertex (i, j) vs (2SP - i, j)
        grid = V[:102].reshape(17, 6, 3)
        left, right = grid[:8], grid[16:8:-1]  # station u and -u
        assert np.allclose(left[:, :, 0], right[:, :, 0], atol=1e-6)
        assert np.allclose(left[:, :, 1], -right[:, :, 1], atol=1e-6)
        assert np.allclose(left[:, :, 2], right[:, :, 2], atol=1e-6)
        assert 0 < V.shape[0] <= 512 and 0 < T.shape[0] <= 900
        assert oracle.fits_print_volume(V)
        mp = oracle.mass_props(genome, V, T)
        assert 0.005 < mp[0] < 0.100
        assert mp[5] > 0 and mp[6] > 0 and mp[7] > 0
        d = oracle.scenario_desc(1000 + i)
        printed, shift = oracle.printed_mass_props(mp, d)
        assert printed[0] > mp[0]
        assert printed[1] > 0 and printed[11] > 0 and printed[15] > 0 and printed[19] > 0
        assert np.linalg.norm(shift) < 0.02


def test_grand_matches_std_mt19937(oracle, tmp_path):
    """The genome draw equals std::mt19937 + uniform_real_distribution<float> (the reference's
    grand(), src/sim.cu:318-321) as built by this host's C++ standard library."""
    lo, hi = oracle.genome_bounds()
    src = tmp_path / "g.cpp"
    src.write_text(r"""
#include <random>
#include <cstdio>
#include <cmath>
int main(int argc, char** argv) {
  float lo[35], hi[35];
  FILE* f = fopen(argv[1], "rb"); fread(lo, 4, 35, f); fread(hi, 4, 35, f); fclose(f);
  std::mt19937 rng(atoi(argv[2])); std::uniform_real_distribution<float> u(0, 1);
  for (int k = 0; k < 300; k++) for (int i = 0; i < 35; i++) {
    float v = lo[i] + u(rng) * (hi[i] - lo[i]);
    v = fminf(hi[i], fmaxf(lo[i], v)); fwrite(&v, 4, 1, stdout); }
}
""")
    exe = tmp_path / "g"
    r = subprocess.run(["g++", "-O2", "-ffp-contract=off", str(src), "-o", str(exe)], capture_output=True)
    if r.returncode != 0:
        pytest.skip("no host C++ compiler")
    bounds = tmp_path / "b.bin"
    bounds.write_bytes(lo.tobytes() + hi.tobytes())
    for seed in (0, 42, 2024):
        out = subprocess.run([str(exe), str(bounds), str(seed)], capture_output=True).stdout
        ref = np.frombuffer(out, np.float32).reshape(300, 35)
        assert np.array_equal(bits(ref), bits(oracle.grand(seed, 300)))


def test_oracle_fp64_agrees_with_fp32_on_geometry(oracle, host_golden):
    for genome in host_golden["genomes"][:20]:
        V32, T = oracle.build_mesh(genome, 32)
        V64, _ = oracle.build_mesh(genome, 64)
        assert np.allclose(V32, V64, rtol=0, atol=2e-7)
        m32 = oracle.mass_props(genome, V32, T, 32)
        m64 = oracle.mass_props(genome, V64, T, 64)
        assert abs(m32[0] - m64[0]) <= 1e-5 * m64[0]                      # mass
        assert np.all(np.abs(m32[2:5] - m64[2:5]) <= 1e-6 * genome[1])    # COM vs chord
        iscale = np.max(m64[5:8])                                         # inertia vs its diagonal
        assert np.all(np.abs(m32[5:11] - m64[5:11]) <= 1e-5 * iscale)
