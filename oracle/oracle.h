/*
 * oracle.h -- CPU restatement of planes-rl's fitness-evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the test oracle of the CUDA path in
 * planes-rl_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it.  The product never links or calls it.
 *
 * It restates, in plain C, the reference's algorithm for this path:
 *   - mesher            src/common.h:124-307  (camber_z, span_yz, wing_pt, emit_*, build_mesh,
 *                                              mesh_extent, fits_print_volume)
 *   - mass_props        src/common.h:309-365
 *   - scenario draw     src/common.h:368-421  (mix_bits, scenario_u01/_signed, scenario_desc)
 *   - print variation   src/common.h:423-457  (point_inertia, invert_inertia, printed_mass_props)
 *   - gust field        src/common.h:459-467  (wind_at)
 *   - panel prepare     src/sim.cu:25-49      (k_prepare)
 *   - release + flight  src/sim.cu:55-212     (k_sim; its 128-thread strided partial sums, warp
 *                                              shuffle tree and serial 4-warp sum are reproduced
 *                                              in that order, as is the 600-step chunk time reset
 *                                              of src/sim.cu:113 driven by src/sim.cu:238-248)
 *   - tail-aware score  src/sim.cu:340-357    (robust_scores)
 *   - genome draw       src/sim.cu:316-321    (grand/gset over std::mt19937 + libstdc++'s
 *                                              uniform_real_distribution<float>)
 *
 * Every function exists in two precisions: orf_* (float, the reference's arithmetic) and ord_*
 * (double, the FP64 re-run used to state the error of every FP32 result).  Model constants are
 * the reference's float literals in both precisions, so the FP64 run differs from the FP32 run
 * only in its arithmetic.
 *
 * Pinning: the float mesher / mass_props / scenario / print-variation / gust functions are
 * checked bit-for-bit against the reference's own src/common.h compiled on the host
 * (oracle/build_ref.py -> oracle/_ref/libref_host.so -> tests/golden/host_golden.npz).
 * The flight step is pinned against the reference's CUDA build run on a GB300
 * (tests/golden/ref_cuda_*.npz, made by tests/golden/make_ref_cuda_golden.py).
 *
 * Layouts (all arrays are flat, caller-allocated):
 *   genome      35 float                         (src/common.h:61-97, 140 B)
 *   V           [MAX_V][3], T [MAX_T][3] int
 *   mass props  20: mass, invmass, com[3], I[6] (xx yy zz xy xz yz), invI[9]
 *   scenario    25: speed pitch yaw roll height roll_rate pitch_rate yaw_rate air_rho skin_cf
 *                   gust base_x base_y force_pitch force_yaw grip_x grip_y grip_z
 *                   material_scale infill_ratio print_bias_x print_bias_y print_bias_z
 *                   warp_pitch warp_roll                         (src/common.h:377-387)
 *   state       16: pos[3], q[4] (w x y z), vel[3], wb[3], t, done, fitness
 *   panels      pc [pop][MAX_T][4] = COM-relative centroid xyz + area
 *               pn [pop][MAX_T][4] = unit normal xyz + 0           (src/sim.cu:40-48)
 */
#ifndef PLANES_ORACLE_H
#define PLANES_ORACLE_H
#include <stdint.h>

#define OR_GENOME_N 35
#define OR_MAX_V 512
#define OR_MAX_T 900
#define OR_MP_N 20
#define OR_SCEN_N 25
#define OR_STATE_N 16
#define OR_SIM_MAX_STEPS 7200
#define OR_CHUNK 600

#ifdef __cplusplus
extern "C" {
#endif

#define OR_DECLARE(P, R)                                                                          \
    int P##build_mesh(const float* genome, R* V, int* T, int* nv, int* nt);                       \
    int P##fits_print_volume(const R* V, int nv);                                                 \
    void P##mesh_extent(const R* V, int nv, R* ext);                                              \
    void P##mass_props(const float* genome, const R* V, const int* T, int nt, R* mp);             \
    void P##scenario_desc(int seed, R* d);                                                        \
    void P##printed_mass_props(const R* mp, const R* d, R* out, R* cg_shift);                     \
    void P##wind_at(const R* p, R t, int seed, R* out);                                           \
    void P##prepare(const float* genomes, int pop, R* pc, R* pn, R* mp, int* nt);                 \
    void P##release(const R* mp_plane, int nt, int env_seed, R* state);                           \
    void P##step(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed,               \
                 const R* state_in, int step, int max_steps, R* state_out, R* FT);                \
    void P##fly(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed, int max_steps, \
                R* fitness, int* steps, R* state_out);                                            \
    void P##fly_rec(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed, int p,        \
                    R spread, int rec_every, int rec_cap, R* rec, R* fitness);                     \
    void P##fly_smooth(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed,         \
                       int max_steps, R* d, int* steps, int* kind);                                \
    void P##eval_batch(const float* genomes, int pop, const int* seeds, int nseeds, int vary,     \
                       int max_steps, R* dist, int* steps, int nthreads);                         \
    void P##eval_prepared(const R* pc, const R* pn, const R* mp, const int* nt, int pop,          \
                          const int* seeds, int nseeds, int vary, int max_steps, R* dist,         \
                          int* steps, int nthreads);

OR_DECLARE(orf_, float)
OR_DECLARE(ord_, double)

/* Tail-aware fitness (src/sim.cu:340-357): 0.65 mean + 0.25 mean(worst ceil(S/4)) + 0.10 min,
 * float arithmetic without contraction (the reference's x86-64 host build). */
void or_robust_scores(const float* samples, int pop, int nseeds, float* scores);

/* Robustness-audit statistics of n distances (src/sim.cu:291-309, percentile src/sim.cu:250-256):
 * out[13] = min p05 p10 p25 median mean sd p75 p90 p95 max CVaR10 failures, float arithmetic
 * without contraction on the ascending-sorted distances (n >= 1). */
void or_audit_stats(const float* dist, int n, float* out);

/* std::mt19937 (seeded like the reference's `std::mt19937 rng(seed)`), and the genome draw of
 * src/sim.cu:318-321: gene i = clamp(G_LO[i] + u * (G_HI[i] - G_LO[i])) with u from
 * uniform_real_distribution<float>(0,1) as libstdc++ computes it (one 32-bit draw). */
void or_grand(uint32_t seed, int n, float* genomes);
void or_mt19937_raw(uint32_t seed, int n, uint32_t* out);
void or_genome_bounds(float* lo, float* hi);

#ifdef __cplusplus
}
#endif
#endif
