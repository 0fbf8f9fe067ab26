// pe_internal.cuh -- argument blocks and launchers shared by the kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pe_model.cuh"

namespace pe {

// Per-plane table written by the prepare kernels, read by the flight kernels.
//   nt[p]   triangles flown (0 when the mesh does not fit the print volume)
//   off[p]  first panel of plane p in the packed panel arrays (exact prefix of topology nt)
//   mp[p]   MassProps, 20 floats (the 3x3 inverse from FP64)
//   ext[p]  mesh extent xyz (metres) and the topology triangle count (as float)
struct PlaneTable {
    int* nt;
    int* off;
    float* mp;
    float4* ext;
};

struct PrepArgs {
    const float* genomes;  // [pop][35]
    int pop;
    int* nt_topo;          // [pop] scratch: topology triangle counts
    int* block_sum;        // [nblocks] scratch: per-block totals, then their exclusive prefix
    PlaneTable pt;
    float4* pc;            // [total] COM-relative centroid xyz + area
    float4* pn;            // [total] unit normal xyz + 0
};

constexpr int kScanBlock = 1024;  // genomes per block of the prefix scan

void launch_prepare(const PrepArgs& a, int* d_total, cudaStream_t s);
// Parity probe: 1 = correctly rounded chordwise stations (default), 0 = run-time quotient.
cudaError_t set_station_mode(int ieee);

// One launch of the flight kernel advances every listed flight by at most
// step_end - step_begin steps.
struct FlightArgs {
    const float4* pc;
    const float4* pn;
    const int* plane_nt;
    const int* plane_off;
    const float* plane_mp;
    const int* seeds;       // [nseeds] device copy of the scenario seeds
    int nseeds;
    int vary;               // env_seed = seeds[s] + (vary ? p * 7919 : 0)
    int max_steps;
    int n_flights;          // pop * nseeds; flight f = p * nseeds + s
    int step_begin, step_end;
    const int* active_in;   // flights to advance (nullptr: all, first launch)
    const int* n_active_in;
    int* active_out;        // flights still airborne after this launch (nullptr: last launch)
    int* n_active_out;
    int* work;              // fetch counter, zero at launch
    FlightState* state;     // [n_flights]
    float* dist;            // [n_flights] fitness per flight (metres; -100 oversize, -10 NaN)
    int* steps;             // [n_flights] integrated steps
    // pose recording and launch grid of the reference's gpu_sim (src/sim.cu:72-79, 115-128);
    // rec == nullptr for every evaluation path
    float* rec;             // [n_flights][rec_cap][8]: pos xyz, q wxyz, alive
    int rec_every, rec_cap;
    float spread;           // launch grid spacing (> 0 offsets the release; flight index = grid index)
    // body frame only: 1 = a flight ended by ground contact reports the z = 0 crossing interpolated
    // between its last two states (the distance pe_grad differentiates) instead of the last x
    int smooth;
    // the forward pass of pe_grad (launch_grad_forward only).  grad_setup holds each flight's
    // constants and release state from the gradient model (kGradSetupFloats per flight, written by
    // pe_grad.cu), so the forward flies the very flight the reverse pass differentiates.  Out: the
    // state every grad_K steps (FlightState layout, the clock restarted at 600-step boundaries as the
    // next step would), every step's body-frame aerodynamic force and torque (grad_fsum may be null)
    // and how the flight ended (0 oversize, 1 ground, 2 other bound or horizon, 3 NaN).
    const float* grad_setup;  // [n_flights][kGradSetupFloats]
    float* grad_ck;           // [n_flights][grad_nck][16]
    float* grad_fsum;         // [n_flights][max_steps][8]: F xyz, tau xyz, 0, 0
    int* grad_kind;           // [n_flights]
    int grad_K, grad_nck;
};

// Per-flight record of the gradient model's set-up, read by pe_grad's forward pass:
//   [0] mass [1] invmass [2..7] I (xx yy zz xy xz yz) [8..16] I^-1 (row-major) [17] skin cf
//   [18] gust phase [19] gust scale [20] base wind x [21] base wind y [22..24] CG shift xyz
//   [25] air density [26] warp pitch [27] warp roll [32..47] release state (FlightState layout)
constexpr int kGradSetupFloats = 48;

// Execution shape of the flight kernel (the autotuner's search space).
struct FlightShape {
    int lanes;        // lanes per flight: 16 or 32
    int warps;        // warps per block
    int chunk;        // steps per launch
    int blocks;       // grid size (0: fill the GPU)
    int fast;         // 0: reference arithmetic (pe_flight.cu), 1: body frame (pe_flight_fast.cu)
    int cap;          // body frame only: 1 = registers capped at 96, 2 = 128 (warps <= 4),
                      // 3 = 184 in one-warp blocks
};

int flight_blocks_per_sm(const FlightShape& sh);
size_t flight_smem_bytes(const FlightShape& sh);
cudaError_t launch_flight(const FlightArgs& a, const FlightShape& sh, int grid, cudaStream_t s);
int flight_fast_blocks_per_sm(const FlightShape& sh);
cudaError_t launch_flight_fast(const FlightArgs& a, const FlightShape& sh, int grid, cudaStream_t s);
// pe_grad's forward pass: the body-frame flight kernel with smoothed landing distances on the
// gradient model's set-up (grad_setup), writing grad_ck, grad_fsum and grad_kind.  One launch over
// every flight (step_begin 0, step_end = max_steps); 32 lanes per flight in 4-warp blocks for at
// most 192 flights per SM, else the evaluation's one-warp shape.
// Shared-memory opt-in and blocks per SM of its two shapes (32-lane, 16-lane), once per engine.
cudaError_t grad_forward_configure(int bps[2]);
cudaError_t launch_grad_forward(const FlightArgs& a, int nsm, const int bps[2], cudaStream_t s);
cudaError_t launch_debug_step_fast(const FlightArgs& a, const FlightState* state_in, FlightState* state_out,
                                   float* FT, int* done, float* fit, int step, int lanes, cudaStream_t s);

// Message returned by pe_last_error() on this thread.
void set_last_error(const char* msg);

// Tail-aware score per plane from dist[pop][nseeds].
cudaError_t launch_scores(const float* dist, int pop, int nseeds, float* scores, cudaStream_t s);

// Teacher-forced single step for parity tests: each flight f starts from state_in[f] (clock
// included) at step `step`, applies one step and writes state_out[f] and FT[f*6..] (aerodynamic
// force and torque sums, world frame).
cudaError_t launch_debug_step(const FlightArgs& a, const FlightState* state_in, FlightState* state_out,
                              float* FT, int* done, float* fit, int step, int lanes, cudaStream_t s);

// Release state of every flight (parity tests).
cudaError_t launch_debug_release(const FlightArgs& a, FlightState* out, cudaStream_t s);

// ---------------------------------------------------------------- gradient (pe_grad.cu)
// Per-flight adjoint of the plane data: mass, I[6], one pad, then SoA over the panels:
// centroid x, y, z, area, normal x, y, z (kNtMax each).
constexpr int kAdjStride = 8 + 7 * kNtMax;
constexpr int kGradMaxSeeds = 256;
constexpr int kGradMaxK = 600;

struct GradArgs {
    const float4* pc;
    const float4* pn;
    const int* plane_nt;
    const int* plane_off;
    const float* plane_mp;
    const float* genomes;  // [pop][35]
    const int* seeds;      // [nseeds]
    int pop, nseeds, vary, max_steps;
    int K;                 // checkpoint interval (steps)
    int nck;               // checkpoints per flight: max_steps / K + 1
    int n_flights;         // pop * nseeds, flight f = p * nseeds + s
    int* work;             // [2] queue counters (forward, reverse), zero at launch
    float* setup;          // [n_flights][kGradSetupFloats] the model's set-up of each flight
    float* ck;             // [n_flights][nck][16] checkpointed states
    float* fsum;           // [n_flights][max_steps][8] each step's body force and torque, written by
                           // the forward pass (nullptr: the reverse pass recomputes them from the panels)
    float* dist;           // [n_flights] smoothed landing distance
    int* steps;            // [n_flights] steps flown
    int* kind;             // [n_flights] 0 oversize, 1 ground, 2 other bound or horizon, 3 NaN
    int* order;            // [n_flights] flights by steps, longest first
    int n_long;            // the first n_long of them take the pipelined reverse pass (needs fsum)
    int group;             // flights per block of the other flights' reverse pass: 1, or
                           // grad_group_size(K) with fsum
    int n_single;          // grouped: the first n_single flights after the n_long take a block each
    float* adj;            // [n_flights][kAdjStride]
    float* ybar;           // [pop][kAdjStride] weighted sum of each plane's flight adjoints
    float* obj;            // [pop] objective (may be null)
    float* grad;           // [pop][35]
};

size_t grad_reverse_smem(int K);
// Grid sizes of the reverse kernels (persistent: blocks per SM x SMs) for checkpoint interval K and
// their shared-memory opt-ins: rev_grid[0] one flight per block, rev_grid[1] grouped (0 when
// grad_group_size(K) is 1).
cudaError_t grad_configure(int K, int rev_grid[2], int nsm);
// Flights per block of the grouped reverse pass at checkpoint interval K (1: not available).
int grad_group_size(int K);
// set-up -> forward (launch_grad_forward with `fwd`) -> order -> [event mid] -> reverse -> weights
// -> genome, on stream s.
// With a.n_long > 0 the longest flights' reverse pass runs pipelined beside the others'; with
// a.group > 1 the others run a.group flights per block.
cudaError_t launch_grad(const GradArgs& a, const FlightArgs& fwd, int nsm, const int fwd_bps[2], const int rev_grid[2],
                        cudaStream_t s, cudaEvent_t mid);
// Whether checkpoint interval K admits the pipelined pass for the longest flights (K <= kPipeMaxK).
bool grad_long_pass(int K);
constexpr int kPipeMaxK = 96;

// ---------------------------------------------------------------- objective only (pe_objective.cu)
// Per-plane data in the objective's precision T: mass, I[6], flown triangle count (as T; 0 when
// the mesh does not fit the print volume), then SoA over the panels: COM-relative centroid x, y,
// z, area, unit normal x, y, z (kNtMax each).
constexpr int kObjPlaneStride = 8 + 7 * kNtMax;

struct ObjArgs {
    const float* genomes;  // [pop][35]
    const int* seeds;      // [nseeds]
    int pop, nseeds, vary, max_steps;
    void* plane;           // [pop][kObjPlaneStride] of float or double
    double* dist;          // [pop * nseeds] smoothed landing distance
    double* obj;           // [pop] objective (may be null)
    int* work;             // queue counter
};
// prepare -> flights -> objective in FP32 (precision 32) or FP64 (64), on stream s.
cudaError_t launch_objective(const ObjArgs& a, int precision, int nsm, cudaStream_t s);

}  // namespace pe
