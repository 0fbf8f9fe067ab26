"""Record golden vectors from the reference's own host code (src/common.h, src/designs.cu).

Run in the container that holds the reference tree:  python tests/golden/make_host_golden.py
It builds oracle/_ref/libref_host.so from the reference sources (oracle/build.py) and writes
tests/golden/host_golden.npz:
  presets          [5][35]   the reference's five preset genomes (write_presets -> seeds.bin)
  genomes          [G][35]   presets + genomes drawn like grand() from std::mt19937(2024)
  nv, nt           [G]       mesh sizes (build_mesh)
  V                [G][241][3], T [G][344][3]   mesh vertices / triangles (zero padded)
  printable        [G]       fits_print_volume(V, 250 mm - wall)
  extent           [G][3]    mesh_extent
  mp               [G][20]   mass_props
  scen_seeds       [K]       seeds incl. negative and overflowing ones
  scen             [K][25]   scenario_desc
  printed, cg      [K][20], [K][3]   printed_mass_props(mp[k % G], scen[k])
  wind_p, wind_t   [K][3], [K] sample points; wind [K][3] = wind_at(p, t, seed)
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle_py  # noqa: E402

obuild = oracle_py._build

NV_MAX, NT_MAX = 241, 344


def main():
    lib_path = obuild.build_ref()
    if lib_path is None:
        raise SystemExit("reference tree not found; golden vectors can only be recorded where it exists")
    ref = C.CDLL(lib_path)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    d = tempfile.mkdtemp()
    ref.ref_write_presets(d.encode())
    raw = open(os.path.join(d, "seeds.bin"), "rb").read()
    n = int(np.frombuffer(raw[:4], np.int32)[0])
    presets = np.frombuffer(raw[4:4 + 140 * n], np.float32).reshape(n, 35).copy()
    genomes = np.concatenate([presets, oracle_py.grand(2024, 43)])
    G = genomes.shape[0]
    nv = np.zeros(G, np.int32); nt = np.zeros(G, np.int32)
    V = np.zeros((G, NV_MAX, 3), np.float32); T = np.zeros((G, NT_MAX, 3), np.int32)
    printable = np.zeros(G, np.int32); extent = np.zeros((G, 3), np.float32); mp = np.zeros((G, 20), np.float32)
    for i in range(G):
        Vb = np.zeros((512, 3), np.float32); Tb = np.zeros((900, 3), np.int32)
        a, b = C.c_int(), C.c_int()
        ref.ref_build_mesh(P(genomes[i]), P(Vb), P(Tb), C.byref(a), C.byref(b))
        nv[i], nt[i] = a.value, b.value
        V[i, :a.value] = Vb[:a.value]; T[i, :b.value] = Tb[:b.value]
        printable[i] = ref.ref_fits_print_volume(P(Vb), a)
        ref.ref_mesh_extent(P(Vb), a, P(extent[i]))
        ref.ref_mass_props(P(genomes[i]), P(Vb), P(Tb), b, P(mp[i]))
    seeds = np.array(list(range(-20, 180)) + [2**31 - 1, -2**31, 100003, 100003 + 127 * 7919,
                                              2930001 + 99999 * 7919, 9001, 123456789, 777, 25, 36],
                     dtype=np.int64).astype(np.int32)
    K = seeds.size
    scen = np.zeros((K, 25), np.float32); printed = np.zeros((K, 20), np.float32); cg = np.zeros((K, 3), np.float32)
    rng = np.random.default_rng(7)
    wind_p = np.stack([rng.uniform(-5, 25, K), rng.uniform(-5, 5, K), rng.uniform(0, 3, K)], 1).astype(np.float32)
    wind_t = rng.uniform(0, 12, K).astype(np.float32)
    wind = np.zeros((K, 3), np.float32)
    for k in range(K):
        ref.ref_scenario_desc(int(seeds[k]), P(scen[k]))
        ref.ref_printed_mass_props(P(mp[k % G]), P(scen[k]), P(printed[k]), P(cg[k]))
        ref.ref_wind_at(P(wind_p[k]), C.c_float(wind_t[k]), int(seeds[k]), P(wind[k]))
    out = os.path.join(HERE, "host_golden.npz")
    np.savez_compressed(out, presets=presets, genomes=genomes, nv=nv, nt=nt, V=V, T=T, printable=printable,
                        extent=extent, mp=mp, scen_seeds=seeds, scen=scen, printed=printed, cg=cg,
                        wind_p=wind_p, wind_t=wind_t, wind=wind)
    print("wrote", out, os.path.getsize(out), "bytes;", G, "genomes,", K, "seeds")


if __name__ == "__main__":
    main()
