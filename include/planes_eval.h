/*
 * planes_eval.h -- C ABI of the GB300 (sm_103a) fitness-evaluation path of planes-rl.
 *
 * Library: planes-rl_gb300/lib/libplanes_gb300.so.  Every entry point returns an int status
 * (PE_OK on success) and never exits the process; pe_last_error() gives the message of the
 * last failure on the calling thread.  Pointers named d_* are device pointers the caller owns,
 * h_* are host pointers.  `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  No torch or other library types cross this boundary.
 *
 * Data formats (identical to the reference):
 *   genome     35 float32, gene order of struct Genome (src/common.h:61-97), 140 B
 *   best.bin   one raw genome (src/sim.cu:327-331)
 *   pop.bin    int32 n, then n genomes (src/sim.cu:333-338, read at src/main.cu:28-34)
 *   fitness    metres flown along +x; -100 for a mesh beyond the 250 mm print volume,
 *              -10 for a flight whose state became NaN (src/sim.cu:109, 198-201)
 */
#ifndef PLANES_EVAL_H
#define PLANES_EVAL_H

#ifdef __cplusplus
extern "C" {
#endif

#define PE_OK 0
#define PE_EINVAL 1   /* bad argument (null pointer, size out of range) */
#define PE_ENOMEM 2   /* device or host allocation failed */
#define PE_ECUDA 3    /* a CUDA call failed; see pe_last_error() */
#define PE_ENOTSUP 4  /* argument combination not implemented */
#define PE_ENODEV 5   /* no CUDA device */

#define PE_GENOME_FLOATS 35
#define PE_MASSPROPS_FLOATS 20  /* mass, invmass, com[3], I[6] (xx yy zz xy xz yz), invI[9] */
#define PE_STATE_FLOATS 16      /* pos[3], q[4] (w x y z), vel[3], wb[3], t, step (int32 bits), pad */
#define PE_MAX_STEPS 7200       /* SIM_MAX_STEPS, src/common.h:471 */
/* Largest population of one call (pe_eval_batch, pe_evaluate_population, pe_grad, pe_objective,
 * pe_autotune, pe_panelbuf_alloc): a plane's panels start at a 32-bit offset into the packed panel
 * set, and 4,194,304 planes of at most 344 panels stay below 2^31.  The reference has no such
 * bound (one block per plane, src/sim.cu:214-218); larger populations go in several calls. */
#define PE_MAX_POP 4194304

/* Message of the last failed call on this thread ("" if none). */
const char* pe_last_error(void);
/* Library ABI version (major * 100 + minor). */
int pe_version(void);

/* ------------------------------------------------------------------------------------------
 * Compatibility layer: the reference's evaluation boundary, src/sim.h:9-13.
 * ---------------------------------------------------------------------------------------- */

/* Replaces `void* panelbuf_alloc(int pop)` (src/sim.h:9, src/sim.cu:220-228).  The handle owns
 * the per-plane panels, mass properties and flight state of up to `pop` planes. */
int pe_panelbuf_alloc(int pop, void** out_pb);

/* Replaces `void panelbuf_free(void* pb)` (src/sim.h:10, src/sim.cu:230-235).  NULL is a no-op. */
int pe_panelbuf_free(void* pb);

/* Replaces `void gpu_prepare(const Genome* d_gs, void* pb, int pop)` (src/sim.h:11,
 * src/sim.cu:214-218): mesh, mass properties, printability and panels of d_genomes[pop].
 * Asynchronous on `stream`. */
int pe_prepare(const float* d_genomes, void* pb, int pop, void* stream);

/* Replaces `void gpu_sim(void* pb, int pop, int seed, float* d_fitness, float8* d_rec,
 * int rec_every, int rec_cap, float spread, int vary_scenarios)` (src/sim.h:12-13,
 * src/sim.cu:238-248): flies plane p under env_seed = seed + (vary_scenarios ? p * 7919 : 0)
 * and writes d_fitness[p].  Returns after the flights completed, as the reference does.
 * Pose recording (src/sim.cu:115-128): with d_rec != NULL (device, [pop][rec_cap][8] floats:
 * pos xyz, q wxyz, alive), every step that is a multiple of rec_every records the pose before
 * it is integrated, at the reference's slot -- each 600-step launch restarts at step0 / rec_every
 * -- while the slot is below rec_cap; a finished or oversize flight keeps being recorded with
 * alive = 0 until step 7199.  launch_spread > 0 places plane p on the reference's showcase grid
 * (src/sim.cu:72-79), which moves its release point and hence its flight.  Both run in the
 * default body-frame shape. */
int pe_sim(void* pb, int pop, int seed, float* d_fitness, float* d_rec, int rec_every, int rec_cap,
           float launch_spread, int vary_scenarios, void* stream);

/* ------------------------------------------------------------------------------------------
 * Batched layer: one call evaluates pop genomes x nseeds scenarios.
 * ---------------------------------------------------------------------------------------- */

typedef struct pe_engine pe_engine;

/* Flight formulation and execution shape.  For a given formulation the results do not depend
 * on lanes, warps, chunk, blocks or use_graph (every sum has one fixed order).
 *   formulation 0: the reference's arithmetic: panels rotated to the world frame, sums in the
 *                  reference's 128-thread order (src/sim.cu:134-176).
 *   formulation 1: the same physics in the body frame, about half the operations per panel;
 *                  results agree with formulation 0 to rounding (the default).
 * In formulation 1, a batch of at most 192 flights per SM (a few waves of flights, bound by the
 * longest ones) flies 32 lanes per flight in 4-warp blocks when lanes = 16, reg_cap = 0 or 3 and
 * blocks = 0: the same results, sooner.
 * Default: lanes 16, warps 1, chunk 7200, blocks 0, use_graph 0, formulation 1, reg_cap 3. */
typedef struct {
    int lanes;       /* lanes per flight: 16 or 32 (formulation 0: 32 only) */
    int warps;       /* warps per block of the flight kernel: 1..8 */
    int chunk;       /* steps per flight launch: 1..7200 */
    int blocks;      /* flight grid size; 0 = fill the GPU (persistent) */
    int use_graph;   /* 1 = replay the whole evaluation from a captured CUDA graph */
    int formulation; /* 0 = reference arithmetic, 1 = body frame */
    int reg_cap;     /* body frame only: registers capped so more flights reside per SM, 1 = 96,
                        2 = 128 (both require warps <= 4), 3 = 184 in one-warp blocks (warps = 1,
                        11 blocks per SM) */
} pe_config;

int pe_engine_create(int device, pe_engine** out);
int pe_engine_destroy(pe_engine* e);
int pe_engine_get_config(const pe_engine* e, pe_config* cfg);
int pe_engine_set_config(pe_engine* e, const pe_config* cfg);

/* Evaluate d_genomes[pop][35] under nseeds scenarios each.  Flight f = p * nseeds + s uses
 * env_seed = h_seeds[s] + (vary ? p * 7919 : 0) (src/sim.cu:64); the reference's GA calls this
 * with vary = 0 and seeds gen*S + s + 1 (src/sim.cu:435), its evaluate/holdout paths with
 * vary = 1 (src/sim.cu:267, 452).  Flights stop at ground contact or at step max_steps - 1
 * (<= 7200).  Outputs (any may be NULL):
 *   d_dist[pop * nseeds]  fitness of each flight, plane-major (the reference's samples layout)
 *   d_steps[pop * nseeds] integrated 600 Hz steps of each flight (0 for oversize meshes)
 *   d_scores[pop]         tail-aware score, src/sim.cu:340-357 (requires nseeds <= 4096)
 * Asynchronous on `stream`; h_seeds is read before the call returns. */
int pe_eval_batch(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                  int max_steps, float* d_dist, int* d_steps, float* d_scores, void* stream);

/* Landing distance of this engine's later evaluations (no reference counterpart): 0 (default)
 * reports the reference's fitness, x after the step that reached the ground (src/sim.cu:198-201);
 * 1 reports the z = 0 crossing interpolated linearly between the flight's last two states, the
 * distance pe_grad differentiates, so that finite differences of pe_eval_batch's scores are
 * differences of pe_grad's objective.  Other endings are unchanged.  Body-frame formulation only
 * (pe_eval_batch returns PE_ENOTSUP otherwise). */
int pe_engine_set_smooth_landing(pe_engine* e, int on);

/* The same evaluation from host buffers (copies in and out included); synchronous. */
int pe_evaluate_population(pe_engine* e, const float* h_genomes, int pop, const int* h_seeds, int nseeds,
                           int vary, int max_steps, float* h_dist, int* h_steps, float* h_scores);

/* Tail-aware fitness of d_samples[pop][nseeds] into d_scores[pop] (src/sim.cu:340-357),
 * bit-identical to the reference's float host reduction.  nseeds <= 4096. */
int pe_robust_scores(const float* d_samples, int pop, int nseeds, float* d_scores, void* stream);

/* Copies of the per-plane results of the last evaluation or prepare (any pointer may be NULL):
 * mass props [pop][20], flown triangle count [pop], panel offset [pop], extent+topology nt
 * [pop][4], panels pc/pn [total][4] in the packed layout. */
int pe_plane_table(pe_engine* e, int pop, float* d_mp, int* d_nt, int* d_off, float* d_ext,
                   float* d_pc, float* d_pn, int* h_total_panels, void* stream);

/* Host copy of one plane of the last evaluation: mass props [20], extent xyz + topology nt [4],
 * flown triangle count (0 = oversize).  Synchronizes the device. */
int pe_plane_info(pe_engine* e, int p, float* h_mp, float* h_ext, int* h_nt);

/* Pick the fastest execution shape on (a sample of) this workload and keep it in the engine.
 * Writes the choice to *best when best != NULL. */
int pe_autotune(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                int max_steps, pe_config* best);

/* Timing of the last pe_eval_batch on this engine, from CUDA events on its stream:
 * ms[0] prepare, ms[1] all flight launches, ms[2] scores; *launches = kernels launched. */
int pe_last_timing(pe_engine* e, float* ms, int* launches);

/* Gradient of each genome's smoothed tail-aware objective with respect to its 35 genes.  The
 * reference has no gradient; this is the differentiation entry point of its evaluation path
 * (the torch.autograd.Function-style forward/backward pair in one call).  Per flight the
 * landing distance is the z = 0 crossing interpolated between the last two states (ground
 * contact ends the flight, src/sim.cu:198-204); other endings keep x (horizon, |y| > 300,
 * x < -50), NaN flights score -10 and oversize meshes -100, both with zero gradient.  The
 * objective is the tail-aware score of src/sim.cu:340-357 over those distances, differentiated
 * through its active set (mean, the worst ceil(S/4), the worst).  Reverse mode runs over each
 * flight with a checkpoint every checkpoint_every steps (0 = 60) and recompute of each segment,
 * forward mode over mesh -> mass_props -> panels.  Topology genes (fin layout, deck gap) get
 * zero.  Arithmetic is FP32 with the printed inertia inverted in FP64.  The forward pass is the
 * evaluation's packed body-frame flight kernel on the gradient model's IEEE set-up of each flight
 * (print variation, scenario, release); it keeps each step's body force and torque (32 B per
 * flight-step) when all of them fit in 4 GiB, so the recompute runs the model's integrator alone;
 * PE_GRAD_STORE_FORCES=0 in the environment recomputes them from the panels instead.  Objectives
 * and distances are bit-identical either way, gradients agree to ~1e-5.
 *   d_genomes [pop][35] (device), h_seeds [nseeds] host, nseeds <= 256, vary and env seeds as
 *   pe_eval_batch, max_steps <= 7200, 1 <= checkpoint_every <= 600.
 *   Outputs (device): d_grad [pop][35] (required), d_obj [pop] and d_dist [pop][nseeds]
 *   (smoothed distances) may be NULL.
 * Asynchronous on `stream`; pe_last_timing then gives ms[0] prepare, ms[1] forward + ordering,
 * ms[2] reverse + genome contraction. */
int pe_grad(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
            int max_steps, int checkpoint_every, float* d_obj, float* d_grad, float* d_dist, void* stream);

/* The objective pe_grad differentiates, from a forward pass only (no reference counterpart).
 * Every stage -- mesh, printability, mass properties, panels, print variation, release, flight --
 * runs in FP32 (precision 32) or FP64 (precision 64), so central differences of it at a step of
 * 1e-4 of a gene's range are limited by the step, not by float rounding of the inputs.  Same
 * genomes, seeds, vary and max_steps rules as pe_grad (nseeds <= 256).  Outputs (device, double,
 * either may be NULL): d_obj [pop] the tail-aware objective, d_dist [pop][nseeds] the smoothed
 * distances (-100 oversize, -10 NaN flights).  Asynchronous on `stream`; pe_last_timing then
 * gives the whole call in ms[0]. */
int pe_objective(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                 int max_steps, int precision, double* d_obj, double* d_dist, void* stream);

/* The k best of d_scores[n] on the device (NaN worst, ties to the lower index), best first:
 * d_idx[k] and, when d_top != NULL, their scores.  1 <= k <= min(n, 4096).  Asynchronous. */
int pe_topk(const float* d_scores, int n, int k, int* d_idx, float* d_top, void* stream);

/* The k best genomes by score, gathered: d_top[k][35] = d_genomes[d_idx[i]] with d_idx[k] as
 * pe_topk gives it (best first).  The step between a generation and its holdout.  Asynchronous. */
int pe_select_top(const float* d_genomes, const float* d_scores, int pop, int k, float* d_top, int* d_idx,
                  void* stream);

/* One generation of the device GA (the operators of pe_evolve below) from d_genomes[pop][35] and
 * their scores into d_next[pop][35] (not aliased): the pop/64 best first, in order, then the
 * children.  Child i of generation gen draws from the counter-based stream (seed, gen, i), so a
 * call is deterministic.  64 <= pop <= 262144.  Asynchronous on `stream`. */
int pe_ga_step(const float* d_genomes, const float* d_scores, int pop, int gen, int gens,
               unsigned long long seed, float* d_next, void* stream);

/* The GA on the device, optionally with gradient polish (the hybrid search).  No reference
 * counterpart as a whole: the operators are run_ga's (src/sim.cu:472-489; elitism pop/64, 5 %
 * fresh draws, 4-way tournaments, blend a ~ U(-0.1, 1.1), mutation 0.25 x N(0,1) x 0.08 range x
 * (1 - 0.6 gen/gens), clamp) on a counter-based random stream instead of std::mt19937, so results
 * differ from pe_run_ga, which stays the parity mode.  Per generation: all genomes fly the
 * training scenarios gen*nseeds + s + 1 (vary 0); with polish_top > 0 the best polish_top genomes
 * then take polish_steps Adam steps (ascent, normalized genome units, learning rate polish_lr) on
 * pe_grad over the same scenarios and are re-scored before selection; the top 8 fly the holdout
 * (holdout_base + i*7919) and the best-ever genome is the best holdout score (src/sim.cu:446-462).
 * The best-ever genome is finally audited on `audit` scenarios audit_base + i*7919. */
typedef struct pe_evolve_config {
    int pop;               /* >= 64 */
    int gens;
    int nseeds;            /* training scenarios per generation, <= 256 */
    unsigned seed;         /* initial population (grand() of std::mt19937(seed)) and operator stream */
    int max_steps;         /* flight horizon, <= 7200 */
    int polish_top;        /* genomes polished per generation (0: plain GA) */
    int polish_steps;      /* Adam steps per generation */
    float polish_lr;       /* Adam learning rate in normalized genome units */
    int polish_max_steps;  /* horizon of the gradient (0: max_steps) */
    int holdout;           /* holdout scenarios of the top 8 (0: none), <= 4096 */
    int holdout_base;
    int audit;             /* audit scenarios of the best-ever genome (0: none), <= 4096 */
    int audit_base;
} pe_evolve_config;
typedef struct pe_evolve_result {
    float best_genome[35];
    float best_holdout;    /* its holdout score */
    int best_gen;
    float audit_score;     /* tail-aware score over the audit scenarios */
    double gpu_seconds;    /* device time of the generations (CUDA events), audit excluded */
    int grad_calls;
} pe_evolve_result;
/* h_history (may be NULL): [gens][5] train best, holdout best of the top 8, mean, p90 score,
 * device seconds since the start at the end of the generation. */
int pe_evolve(pe_engine* e, const pe_evolve_config* cfg, float* h_history, pe_evolve_result* out);

/* pe_eval_batch without any allocation.  No counterpart in the reference: it exists for callers
 * that cannot allocate device memory when they evaluate (a host whose device memory is all
 * reserved by its own pool, a real-time loop that must not enter the driver's allocator).  Same
 * arguments and results as pe_eval_batch with the default body-frame formulation, on the current
 * device; all working memory is one static device array of about 2.9 MB that every GPU loading
 * the library keeps until exit.  Limits: pop <= 256 and pop * nseeds <= 4096 (PE_EINVAL beyond).
 * The first call on a device looks up that array's address, keeps it for the life of the process
 * (do not cudaDeviceReset that device afterwards), and should precede any stream capture.  All
 * calls share the array and leave their contents in it; calls that overlap on the GPU race and
 * must be serialized by the caller. */
int pe_eval_batch_noalloc(const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                          int max_steps, float* d_dist, int* d_steps, float* d_scores, void* stream);

/* ------------------------------------------------------------------------------------------
 * Host side of the evolve / evaluate call surface.
 * ---------------------------------------------------------------------------------------- */

/* Genome clamp bounds G_LO / G_HI (src/common.h:98-103), 35 floats each. */
int pe_genome_bounds(float* lo, float* hi);
/* n genomes drawn like the reference's grand() from std::mt19937(seed) (src/sim.cu:318-321). */
int pe_random_genomes(unsigned seed, int n, float* h_out);
/* Clamp to the bounds in place (the reference's sanitize(), src/sim.cu:323-325). */
int pe_sanitize_genomes(float* h_genomes, int n);
/* best.bin: one raw genome (src/sim.cu:327-331, src/main.cu:22-26). */
int pe_save_best(const char* path, const float* genome);
int pe_load_best(const char* path, float* genome);
/* pop.bin / archive.bin: int32 n + n genomes (src/sim.cu:333-338, src/main.cu:28-34).  Loads at
 * most cap genomes and reports the file's count in *n_out; a truncated file is PE_EINVAL. */
int pe_save_genomes(const char* path, const float* genomes, int n);
int pe_load_genomes(const char* path, float* genomes, int cap, int* n_out);

/* Robustness-audit statistics of n landing distances on the device (src/sim.cu:291-309; percentile
 * src/sim.cu:250-256), PE_AUDIT_STATS floats: min p05 p10 p25 median mean sd p75 p90 p95 max
 * CVaR10 failures.  The distances are sorted on the device and every sum is taken in ascending
 * order with IEEE rounding, as the reference's host loop does, so each statistic equals its result
 * bit for bit.  1 <= n <= 2^26; d_stats is a device array; enqueued on `stream`. */
#define PE_AUDIT_STATS 13
int pe_distance_stats(const float* d_dist, int n, float* d_stats, void* stream);

/* evaluate_design's flights and audit in one call: one genome (host) under n scenarios with the
 * host seeds (env_seed = seeds[i]), distances kept on the device; h_stats = the PE_AUDIT_STATS
 * statistics of pe_distance_stats; h_dist (optional, n floats) receives the distances (the
 * telemetry CSV needs them).  Blocking. */
int pe_audit(pe_engine* e, const float* h_genome, const int* h_seeds, int n, float* h_stats, float* h_dist);

/* The reference's drivers on the batched engine (device 0):
 *  evaluate_design (src/sim.cu:258-312): one genome x max(8, scenarios) scenarios with
 *    env_seed = base_seed + i * 7919; writes the telemetry CSV (same columns and formats) and prints
 *    the robustness audit; stats (optional, 18 floats) = min p05 p10 p25 median mean sd p75 p90 p95
 *    max CVaR10 failures mass ext_x ext_y ext_z scenarios.
 *  select_finalist (src/sim.cu:359-391): every candidate under the same scenarios (one batch),
 *    finalist-selection.csv and best-final.bin in out_dir.
 *  run_ga (src/sim.cu:393-520): the GA with the reference's std::mt19937(42) stream, holdout of the
 *    top 8 on 128 scenarios, history.csv, checkpoints, pop.bin / archive.bin / best.bin. */
int pe_evaluate_design(const float* genome, int scenarios, int base_seed, const char* csv_path, float* stats);
int pe_select_finalist(const float* candidates, int count, int scenarios, int base_seed, const char* out_dir,
                       int* best_index);
int pe_run_ga(int pop, int gens, int nseeds, const char* out_dir, const char* init_path);

/* Measured FP32 FMA throughput of `device` in TFLOP/s (the flight kernel's roofline peak). */
int pe_fp32_peak_probe(int device, float* tflops);

/* ------------------------------------------------------------------------------------------
 * Parity probes (teacher-forced single steps).  State layout: PE_STATE_FLOATS per flight.
 * ---------------------------------------------------------------------------------------- */

/* Release state of each flight (src/sim.cu:79-107) for the genomes of the last prepare. */
int pe_debug_release(pe_engine* e, int pop, const int* h_seeds, int nseeds, int vary, float* d_state_out,
                     void* stream);

/* One step of every flight from d_state_in at step index `step` (clock restart applied), in the
 * engine's current formulation:
 * d_state_out, d_FT[flight][6] = aerodynamic force and torque sums (world frame, gravity
 * excluded), d_done[flight], d_fit[flight]. */
int pe_debug_step(pe_engine* e, int pop, const int* h_seeds, int nseeds, int vary, int max_steps,
                  const float* d_state_in, float* d_state_out, float* d_FT, int* d_done, float* d_fit,
                  int step, int lanes, void* stream);

/* Mesher probe: 1 (default) evaluates the chordwise stations j/5 and j/3 of the wing grid and
 * keel as correctly rounded quotients, 0 as run-time fast-math quotients.  Process-wide. */
int pe_debug_station_mode(int ieee);

/* Host-side fault injection for the drivers' error paths (no reference counterpart; the
 * reference exits on any CUDA error, src/sim.cu:11-12): after `after_calls` more successful
 * calls, every pe_evaluate_population call fails with PE_ECUDA and the message "injected
 * evaluation failure" before it touches the device.  A negative value switches it off (the
 * default).  Process-wide. */
int pe_debug_fail_evaluations(int after_calls);

#ifdef __cplusplus
}
#endif
#endif
