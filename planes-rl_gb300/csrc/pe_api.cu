// pe_api.cu -- the C ABI of include/planes_eval.h: engine, evaluation pipeline, CUDA-graph
// replay, autotuner, the reference-compatible panelbuf layer and the parity probes.
//
// One evaluation is, on one stream:
//   prepare (3 kernels) -> memset of the launch counters -> ceil(max_steps / chunk) flight
//   launches (persistent grid; each reads the previous launch's list of airborne flights) ->
//   scores.  With use_graph the whole sequence is captured once per shape and replayed.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "../../include/planes_eval.h"
#include "pe_internal.cuh"

using namespace pe;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define PE_CUDA(x)                                                                                  \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess) {                                                                    \
            (void)cudaGetLastError(); /* reported here: do not leave it pending for the next call */ \
            return fail(PE_ECUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                           \
    } while (0)

// A device buffer owned by the engine; freed when the engine is deleted (on the engine's device,
// which pe_engine_destroy selects first), so no buffer can be left out of the teardown.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t m = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc(&p, m * sizeof(T));
        if (e == cudaSuccess) cap = m;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct GraphKey {
    const float* genomes = nullptr;
    float* dist = nullptr;
    int* steps = nullptr;
    float* scores = nullptr;
    cudaStream_t stream = nullptr;
    int pop = -1, nseeds = -1, vary = -1, max_steps = -1, smooth = -1;
    pe_config cfg{};
    bool operator==(const GraphKey& o) const {
        return genomes == o.genomes && dist == o.dist && steps == o.steps && scores == o.scores &&
               stream == o.stream && pop == o.pop && nseeds == o.nseeds && vary == o.vary &&
               max_steps == o.max_steps && smooth == o.smooth && cfg.lanes == o.cfg.lanes && cfg.warps == o.cfg.warps &&
               cfg.chunk == o.cfg.chunk && cfg.blocks == o.cfg.blocks && cfg.formulation == o.cfg.formulation &&
               cfg.reg_cap == o.cfg.reg_cap;
    }
};

bool valid_config(const pe_config& c) {
    return (c.lanes == 16 || c.lanes == 32) && c.warps >= 1 && c.warps <= 8 && c.chunk >= 1 &&
           c.chunk <= kMaxSteps && c.blocks >= 0 && (c.warps * 32) % c.lanes == 0 &&
           (c.formulation == 0 || c.formulation == 1) && (c.use_graph == 0 || c.use_graph == 1) &&
           !(c.formulation == 0 && c.lanes != 32) &&  // the reference arithmetic runs one flight per warp
           (c.reg_cap == 0 || ((c.reg_cap == 1 || c.reg_cap == 2) && c.formulation == 1 && c.warps <= 4) ||
            (c.reg_cap == 3 && c.formulation == 1 && c.warps == 1));
}

}  // namespace

namespace pe {
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace pe

struct pe_engine {
    int device = 0;
    int nsm = 0;
    pe_config cfg{16, 1, 7200, 0, 0, 1, 3};  // fastest shape measured at 100k x 12 on GB300
    int smooth = 0;                          // pe_engine_set_smooth_landing
    // plane table + panels of the last prepare
    DevBuf<int> nt, off, nt_topo, block_sum, total;
    DevBuf<float> mp;
    DevBuf<float4> ext, pc, pn;
    int prepared_pop = 0;
    // flights
    DevBuf<int> seeds, list0, list1, counters;
    DevBuf<FlightState> state;
    DevBuf<float> dist_tmp;
    DevBuf<int> steps_tmp;
    // host-buffer path
    DevBuf<float> g_dev, dist_dev, scores_dev;
    DevBuf<int> steps_dev;
    DevBuf<float> audit_stats;  // pe_audit's 13 statistics
    // timing
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int last_launches = 0;
    bool timed = false;
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    GraphKey gkey;
    // occupancy cache
    int bps_cache[2][4][2][9] = {};
    // gradient
    DevBuf<float> g_setup, g_ck, g_adj, g_ybar, g_dist, g_fsum;
    DevBuf<int> g_steps, g_kind, g_order, g_work;
    int g_K = 0, g_rev_grid[2] = {0, 0}, g_fwd_bps[2] = {0, 0};
    // objective only
    DevBuf<double> o_plane, o_dist;
    DevBuf<int> o_work;
};

namespace {

int ensure_device(pe_engine* e) {
    PE_CUDA(cudaSetDevice(e->device));
    return PE_OK;
}

// The cached graph holds the addresses of the engine's buffers: it is dropped whenever any of them
// moves (grown by a larger call of another entry point, or freed by a failed allocation), so a
// later replay with an unchanged key never touches freed memory.
void drop_graph(pe_engine* e) {
    if (e->gexec) {
        cudaGraphExecDestroy(e->gexec);
        e->gexec = nullptr;
    }
}
struct BufSig {
    const void* p[16];
    bool operator!=(const BufSig& o) const { return memcmp(p, o.p, sizeof p) != 0; }
};
BufSig buf_sig(const pe_engine* e) {
    return BufSig{{e->nt.p, e->off.p, e->nt_topo.p, e->block_sum.p, e->total.p, e->counters.p, e->mp.p, e->ext.p,
                   e->pc.p, e->pn.p, e->list0.p, e->list1.p, e->state.p, e->dist_tmp.p, e->steps_tmp.p,
                   e->seeds.p}};
}

int engine_reserve_buffers(pe_engine* e, int pop, int nflights) {
    const size_t P = (size_t)pop;
    PE_CUDA(e->nt.ensure(P));
    PE_CUDA(e->off.ensure(P));
    PE_CUDA(e->nt_topo.ensure(P));
    PE_CUDA(e->block_sum.ensure(P / kScanBlock + 2));
    PE_CUDA(e->total.ensure(1));
    PE_CUDA(e->counters.ensure((size_t)2 * kMaxSteps + 1));  // enough for any chunk length
    PE_CUDA(e->mp.ensure(P * kMpN));
    PE_CUDA(e->ext.ensure(P));
    PE_CUDA(e->pc.ensure(P * kNtMax));
    PE_CUDA(e->pn.ensure(P * kNtMax));
    if (nflights > 0) {
        const size_t F = (size_t)nflights;
        PE_CUDA(e->list0.ensure(F));
        PE_CUDA(e->list1.ensure(F));
        PE_CUDA(e->state.ensure(F));
        PE_CUDA(e->dist_tmp.ensure(F));
        PE_CUDA(e->steps_tmp.ensure(F));
    }
    return PE_OK;
}

int engine_reserve(pe_engine* e, int pop, int nflights) {
    const BufSig before = buf_sig(e);
    const int rc = engine_reserve_buffers(e, pop, nflights);
    if (buf_sig(e) != before) drop_graph(e);
    return rc;
}

int blocks_for(pe_engine* e, const pe_config& c) {
    if (c.blocks > 0) return c.blocks;
    int& bps = e->bps_cache[c.formulation][c.reg_cap][c.lanes == 16 ? 0 : 1][c.warps];
    if (bps == 0) {
        FlightShape sh{c.lanes, c.warps, c.chunk, 0, c.formulation, c.reg_cap};
        bps = c.formulation ? flight_fast_blocks_per_sm(sh) : flight_blocks_per_sm(sh);
        if (bps <= 0) bps = 1;
    }
    return bps * e->nsm;
}

PrepArgs prep_args(pe_engine* e, const float* d_genomes, int pop) {
    PrepArgs a;
    a.genomes = d_genomes;
    a.pop = pop;
    a.nt_topo = e->nt_topo.p;
    a.block_sum = e->block_sum.p;
    a.pt.nt = e->nt.p;
    a.pt.off = e->off.p;
    a.pt.mp = e->mp.p;
    a.pt.ext = e->ext.p;
    a.pc = e->pc.p;
    a.pn = e->pn.p;
    return a;
}

FlightArgs flight_args(pe_engine* e, int pop, int nseeds, int vary, int max_steps, float* dist, int* steps) {
    FlightArgs a{};
    a.pc = e->pc.p;
    a.pn = e->pn.p;
    a.plane_nt = e->nt.p;
    a.plane_off = e->off.p;
    a.plane_mp = e->mp.p;
    a.seeds = e->seeds.p;
    a.nseeds = nseeds;
    a.vary = vary;
    a.max_steps = max_steps;
    a.n_flights = pop * nseeds;
    a.state = e->state.p;
    a.dist = dist;
    a.steps = steps;
    a.smooth = e->smooth;
    return a;
}

// Enqueue the flights of pop x nseeds (plane table already prepared on this stream).
int enqueue_fly(pe_engine* e, int pop, int nseeds, int vary, int max_steps, float* dist, int* steps,
                cudaStream_t s, int* launches) {
    pe_config c = e->cfg;
    // A batch of at most 192 flights per SM (a holdout of 8 x 128, 1,024 x 8 genomes) flies 32
    // lanes per flight in 4-warp blocks: with few waves of flights the run is bound by its longest
    // flights, whose steps finish sooner at 32 lanes (measured on GB300: 15-23 % faster below 160
    // flights per SM, even near 215, 16 lanes ahead from 320).  The body-frame kernel's results do
    // not depend on the shape.
    if (c.formulation == 1 && c.lanes == 16 && (c.reg_cap == 0 || c.reg_cap == 3) && c.blocks == 0 &&
        (long long)pop * nseeds <= 192LL * e->nsm) {
        c.lanes = 32;
        c.warps = 4;
        c.reg_cap = 0;
    }
    const int nchunks = (max_steps + c.chunk - 1) / c.chunk;
    int* work = e->counters.p;
    int* nact = e->counters.p + nchunks;
    PE_CUDA(cudaMemsetAsync(e->counters.p, 0, sizeof(int) * (2 * nchunks + 1), s));
    FlightShape sh{c.lanes, c.warps, c.chunk, c.blocks, c.formulation, c.reg_cap};
    const int grid = blocks_for(e, c);
    FlightArgs a = flight_args(e, pop, nseeds, vary, max_steps, dist, steps);
    for (int k = 0; k < nchunks; k++) {
        a.step_begin = k * c.chunk;
        a.step_end = std::min((k + 1) * c.chunk, max_steps);
        a.active_in = k == 0 ? nullptr : (k % 2 == 1 ? e->list0.p : e->list1.p);
        a.n_active_in = &nact[k];
        a.active_out = k == nchunks - 1 ? nullptr : (k % 2 == 0 ? e->list0.p : e->list1.p);
        a.n_active_out = &nact[k + 1];
        a.work = &work[k];
        PE_CUDA(c.formulation ? launch_flight_fast(a, sh, grid, s) : launch_flight(a, sh, grid, s));
        (*launches)++;
    }
    return PE_OK;
}

// Inside a stream capture an event record must be an external node to time the replay;
// outside a capture that flag is an error.
cudaError_t record_event(cudaEvent_t ev, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t err = cudaStreamIsCapturing(s, &cs);
    if (err != cudaSuccess) return err;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, s);
}

int enqueue_eval(pe_engine* e, const float* d_genomes, int pop, int nseeds, int vary, int max_steps,
                 float* dist, int* steps, float* scores, cudaStream_t s, int* launches) {
    PE_CUDA(record_event(e->ev[0], s));
    launch_prepare(prep_args(e, d_genomes, pop), e->total.p, s);
    PE_CUDA(cudaGetLastError());
    *launches += 3;
    PE_CUDA(record_event(e->ev[1], s));
    int rc = enqueue_fly(e, pop, nseeds, vary, max_steps, dist, steps, s, launches);
    if (rc != PE_OK) return rc;
    PE_CUDA(record_event(e->ev[2], s));
    if (scores) {
        PE_CUDA(launch_scores(dist, pop, nseeds, scores, s));
        (*launches)++;
    }
    PE_CUDA(record_event(e->ev[3], s));
    return PE_OK;
}

int check_seeds(const int* h_seeds, int nseeds) {
    if (!h_seeds || nseeds <= 0) return fail(PE_EINVAL, "seeds must be a non-empty host array");
    return PE_OK;
}

// Host-side fault injection for the drivers' error paths (pe_debug_fail_evaluations): the number of
// pe_evaluate_population calls still allowed to succeed, or -1 for no injection.
std::atomic<int> g_eval_budget{-1};

// Panel offsets are 32-bit: PE_MAX_POP planes of at most 344 panels stay below 2^31.
int check_pop(int pop) {
    if (pop <= 0 || pop > PE_MAX_POP) return fail(PE_EINVAL, "pop must be in 1..%d (got %d)", PE_MAX_POP, pop);
    return PE_OK;
}

int upload_seeds(pe_engine* e, const int* h_seeds, int nseeds, cudaStream_t s) {
    const void* before = e->seeds.p;
    const cudaError_t grown = e->seeds.ensure((size_t)nseeds);
    if (e->seeds.p != before) drop_graph(e);
    PE_CUDA(grown);
    // pageable source: the call returns once the values are staged, so the caller's array is free
    PE_CUDA(cudaMemcpyAsync(e->seeds.p, h_seeds, sizeof(int) * nseeds, cudaMemcpyHostToDevice, s));
    return PE_OK;
}

}  // namespace

extern "C" {

const char* pe_last_error(void) { return g_err.c_str(); }
int pe_version(void) { return 100; }

int pe_engine_create(int device, pe_engine** out) {
    if (!out) return fail(PE_EINVAL, "out is NULL");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return fail(PE_ENODEV, "no CUDA device");
    if (device < 0 || device >= n) return fail(PE_EINVAL, "device %d out of range (%d devices)", device, n);
    pe_engine* e = new pe_engine();
    e->device = device;
    cudaError_t err = cudaSetDevice(device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, device);
    for (int i = 0; i < 4 && err == cudaSuccess; i++) err = cudaEventCreate(&e->ev[i]);
    if (err != cudaSuccess) {
        pe_engine_destroy(e);
        return fail(PE_ECUDA, "engine init: %s", cudaGetErrorString(err));
    }
    *out = e;
    return PE_OK;
}

int pe_engine_destroy(pe_engine* e) {
    if (!e) return PE_OK;
    cudaSetDevice(e->device);
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    for (int i = 0; i < 4; i++)
        if (e->ev[i]) cudaEventDestroy(e->ev[i]);

    delete e;  // every DevBuf member frees its memory
    return PE_OK;
}

int pe_engine_get_config(const pe_engine* e, pe_config* cfg) {
    if (!e || !cfg) return fail(PE_EINVAL, "NULL argument");
    *cfg = e->cfg;
    return PE_OK;
}

int pe_engine_set_config(pe_engine* e, const pe_config* cfg) {
    if (!e || !cfg) return fail(PE_EINVAL, "NULL argument");
    if (!valid_config(*cfg))
        return fail(PE_EINVAL, "invalid config lanes=%d warps=%d chunk=%d blocks=%d", cfg->lanes, cfg->warps,
                    cfg->chunk, cfg->blocks);
    e->cfg = *cfg;
    return PE_OK;
}

int pe_engine_set_smooth_landing(pe_engine* e, int on) {
    if (!e) return fail(PE_EINVAL, "NULL engine");
    if (on != 0 && on != 1) return fail(PE_EINVAL, "smooth landing is 0 or 1 (got %d)", on);
    e->smooth = on;
    return PE_OK;
}

int pe_eval_batch(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                  int max_steps, float* d_dist, int* d_steps, float* d_scores, void* stream) {
    if (!e || !d_genomes) return fail(PE_EINVAL, "NULL engine or genomes");
    if (e->smooth && e->cfg.formulation != 1)
        return fail(PE_ENOTSUP, "smooth landing distances need the body-frame formulation");
    if (int rc = check_pop(pop)) return rc;
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (max_steps < 1 || max_steps > kMaxSteps) return fail(PE_EINVAL, "max_steps must be in 1..%d", kMaxSteps);
    if ((long long)pop * nseeds > (1LL << 30)) return fail(PE_EINVAL, "pop * nseeds too large");
    if (d_scores && nseeds > 4096) return fail(PE_EINVAL, "scores need nseeds <= 4096");
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nf = pop * nseeds;
    if (int rc = engine_reserve(e, pop, nf)) return rc;
    float* dist = d_dist ? d_dist : e->dist_tmp.p;
    int* steps = d_steps ? d_steps : e->steps_tmp.p;
    if (int rc = upload_seeds(e, h_seeds, nseeds, s)) return rc;
    int launches = 0;
    if (e->cfg.use_graph) {
        GraphKey k;
        k.genomes = d_genomes; k.dist = dist; k.steps = steps; k.scores = d_scores; k.stream = s;
        k.pop = pop; k.nseeds = nseeds; k.vary = vary; k.max_steps = max_steps; k.smooth = e->smooth; k.cfg = e->cfg;
        if (!e->gexec || !(k == e->gkey)) {
            blocks_for(e, e->cfg);  // occupancy query outside the capture
            if (e->gexec) { cudaGraphExecDestroy(e->gexec); e->gexec = nullptr; }
            cudaStream_t cs = s;
            bool own = false;
            if (!cs) {  // the legacy default stream cannot be captured: capture on a private one
                PE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                own = true;
            }
            PE_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            int cl = 0;
            int rc = enqueue_eval(e, d_genomes, pop, nseeds, vary, max_steps, dist, steps, d_scores, cs, &cl);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(cs, &g);
            if (own) cudaStreamDestroy(cs);
            if (rc != PE_OK) { if (g) cudaGraphDestroy(g); return rc; }
            if (ce != cudaSuccess) return fail(PE_ECUDA, "graph capture: %s", cudaGetErrorString(ce));
            ce = cudaGraphInstantiate(&e->gexec, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) { e->gexec = nullptr; return fail(PE_ECUDA, "graph instantiate: %s", cudaGetErrorString(ce)); }
            e->gkey = k;
        }
        PE_CUDA(cudaGraphLaunch(e->gexec, s));
        launches = 3 + (max_steps + e->cfg.chunk - 1) / e->cfg.chunk + (d_scores ? 1 : 0);
    } else {
        if (int rc = enqueue_eval(e, d_genomes, pop, nseeds, vary, max_steps, dist, steps, d_scores, s, &launches))
            return rc;
    }
    e->last_launches = launches;
    e->prepared_pop = pop;
    e->timed = true;
    return PE_OK;
}

int pe_evaluate_population(pe_engine* e, const float* h_genomes, int pop, const int* h_seeds, int nseeds,
                           int vary, int max_steps, float* h_dist, int* h_steps, float* h_scores) {
    if (!e || !h_genomes) return fail(PE_EINVAL, "NULL engine or genomes");
    if (int rc = check_pop(pop)) return rc;
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    for (int b = g_eval_budget.load(); b >= 0; b = g_eval_budget.load()) {
        if (b == 0) return fail(PE_ECUDA, "injected evaluation failure (pe_debug_fail_evaluations)");
        if (g_eval_budget.compare_exchange_weak(b, b - 1)) break;
    }
    if (int rc = ensure_device(e)) return rc;
    const size_t nf = (size_t)pop * nseeds;
    PE_CUDA(e->g_dev.ensure((size_t)pop * kGenomeN));
    PE_CUDA(e->dist_dev.ensure(nf));
    PE_CUDA(e->steps_dev.ensure(nf));
    PE_CUDA(e->scores_dev.ensure((size_t)pop));
    cudaStream_t s = nullptr;
    PE_CUDA(cudaMemcpyAsync(e->g_dev.p, h_genomes, sizeof(float) * kGenomeN * pop, cudaMemcpyHostToDevice, s));
    int rc = pe_eval_batch(e, e->g_dev.p, pop, h_seeds, nseeds, vary, max_steps, e->dist_dev.p, e->steps_dev.p,
                           h_scores ? e->scores_dev.p : nullptr, s);
    if (rc != PE_OK) return rc;
    if (h_dist) PE_CUDA(cudaMemcpyAsync(h_dist, e->dist_dev.p, sizeof(float) * nf, cudaMemcpyDeviceToHost, s));
    if (h_steps) PE_CUDA(cudaMemcpyAsync(h_steps, e->steps_dev.p, sizeof(int) * nf, cudaMemcpyDeviceToHost, s));
    if (h_scores) PE_CUDA(cudaMemcpyAsync(h_scores, e->scores_dev.p, sizeof(float) * pop, cudaMemcpyDeviceToHost, s));
    PE_CUDA(cudaStreamSynchronize(s));
    return PE_OK;
}

int pe_audit(pe_engine* e, const float* h_genome, const int* h_seeds, int n, float* h_stats, float* h_dist) {
    if (!e || !h_genome || !h_stats) return fail(PE_EINVAL, "NULL engine, genome or statistics");
    if (int rc = check_seeds(h_seeds, n)) return rc;
    if (n > (1 << 26)) return fail(PE_EINVAL, "pe_audit takes at most 2^26 scenarios (got %d)", n);
    if (int rc = ensure_device(e)) return rc;
    PE_CUDA(e->g_dev.ensure(kGenomeN));
    PE_CUDA(e->dist_dev.ensure((size_t)n));
    PE_CUDA(e->audit_stats.ensure(PE_AUDIT_STATS));
    cudaStream_t s = nullptr;
    PE_CUDA(cudaMemcpyAsync(e->g_dev.p, h_genome, sizeof(float) * kGenomeN, cudaMemcpyHostToDevice, s));
    if (int rc = pe_eval_batch(e, e->g_dev.p, 1, h_seeds, n, 0, kMaxSteps, e->dist_dev.p, nullptr, nullptr, s))
        return rc;
    if (int rc = pe_distance_stats(e->dist_dev.p, n, e->audit_stats.p, s)) return rc;
    PE_CUDA(cudaMemcpyAsync(h_stats, e->audit_stats.p, sizeof(float) * PE_AUDIT_STATS, cudaMemcpyDeviceToHost, s));
    if (h_dist) PE_CUDA(cudaMemcpyAsync(h_dist, e->dist_dev.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    PE_CUDA(cudaStreamSynchronize(s));
    return PE_OK;
}

int pe_grad(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
            int max_steps, int checkpoint_every, float* d_obj, float* d_grad, float* d_dist, void* stream) {
    if (!e || !d_genomes || !d_grad) return fail(PE_EINVAL, "NULL engine, genomes or gradient");
    if (int rc = check_pop(pop)) return rc;
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (nseeds > kGradMaxSeeds) return fail(PE_EINVAL, "pe_grad takes at most %d seeds", kGradMaxSeeds);
    if (max_steps < 1 || max_steps > kMaxSteps) return fail(PE_EINVAL, "max_steps must be in 1..%d", kMaxSteps);
    const int K = checkpoint_every == 0 ? 60 : checkpoint_every;
    if (K < 1 || K > kGradMaxK) return fail(PE_EINVAL, "checkpoint_every must be in 1..%d", kGradMaxK);
    if ((long long)pop * nseeds > (1LL << 24) || (long long)pop * kGenomeN > (1LL << 30))
        return fail(PE_EINVAL, "pop * nseeds too large for pe_grad");
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nf = pop * nseeds;
    const int nck = max_steps / K + 1;
    if (int rc = engine_reserve(e, pop, 0)) return rc;
    if (e->g_K != K) {
        PE_CUDA(grad_configure(K, e->g_rev_grid, e->nsm));
        if (!e->g_fwd_bps[0]) PE_CUDA(grad_forward_configure(e->g_fwd_bps));
        e->g_K = K;
    }
    PE_CUDA(e->g_setup.ensure((size_t)nf * kGradSetupFloats));
    PE_CUDA(e->g_ck.ensure((size_t)nf * nck * 16));
    PE_CUDA(e->g_adj.ensure((size_t)nf * kAdjStride));
    PE_CUDA(e->g_ybar.ensure((size_t)pop * kAdjStride));
    PE_CUDA(e->g_steps.ensure((size_t)nf));
    PE_CUDA(e->g_kind.ensure((size_t)nf));
    PE_CUDA(e->g_order.ensure((size_t)nf));
    PE_CUDA(e->g_work.ensure(2));
    if (!d_dist) PE_CUDA(e->g_dist.ensure((size_t)nf));
    // Every step's body force and torque from the forward pass (32 B per flight-step), so the
    // reverse pass recomputes states through the integrator alone, when they fit in 4 GiB;
    // PE_GRAD_STORE_FORCES=0 in the environment recomputes them from the panels instead (the same
    // forward outputs bit for bit, gradients to ~1e-5).
    const size_t fsum_floats = (size_t)nf * (size_t)max_steps * 8;
    const char* store_env = getenv("PE_GRAD_STORE_FORCES");
    const bool store_forces = fsum_floats * sizeof(float) <= (4ull << 30) && !(store_env && store_env[0] == '0');
    if (store_forces) PE_CUDA(e->g_fsum.ensure(fsum_floats));
    if (int rc = upload_seeds(e, h_seeds, nseeds, s)) return rc;
    GradArgs a{};
    a.pc = e->pc.p;
    a.pn = e->pn.p;
    a.plane_nt = e->nt.p;
    a.plane_off = e->off.p;
    a.plane_mp = e->mp.p;
    a.genomes = d_genomes;
    a.seeds = e->seeds.p;
    a.pop = pop;
    a.nseeds = nseeds;
    a.vary = vary;
    a.max_steps = max_steps;
    a.K = K;
    a.nck = nck;
    a.n_flights = nf;
    a.work = e->g_work.p;
    a.setup = e->g_setup.p;
    a.ck = e->g_ck.p;
    a.fsum = store_forces ? e->g_fsum.p : nullptr;
    a.dist = d_dist ? d_dist : e->g_dist.p;
    a.steps = e->g_steps.p;
    a.kind = e->g_kind.p;
    a.order = e->g_order.p;
    a.adj = e->g_adj.p;
    a.ybar = e->g_ybar.p;
    a.obj = d_obj;
    a.grad = d_grad;
    PE_CUDA(record_event(e->ev[0], s));
    launch_prepare(prep_args(e, d_genomes, pop), e->total.p, s);
    PE_CUDA(cudaGetLastError());
    PE_CUDA(record_event(e->ev[1], s));
    // the forward pass: the evaluation's body-frame kernel on the model's set-up records, smoothed
    // distances, checkpoints and per-step forces
    FlightArgs fa = flight_args(e, pop, nseeds, vary, max_steps, a.dist, a.steps);
    fa.smooth = 1;
    fa.step_begin = 0;
    fa.step_end = max_steps;
    fa.work = a.work;
    fa.grad_setup = a.setup;
    fa.grad_ck = a.ck;
    fa.grad_fsum = a.fsum;
    fa.grad_kind = a.kind;
    fa.grad_K = K;
    fa.grad_nck = nck;
    // The reverse pass is bound by its longest flights' chains and by how many flights it keeps in
    // flight.  With the stored forces the flights other than the longest take grad_group_size(K) per
    // block, warp 0 carrying all their integrator chains at once: the longest take the pipelined
    // pass (one per 8 SMs, one per 4 SMs in a batch of at most 4 flights per SM such as the GA's
    // polish of 64 genomes x 8 scenarios), the next nsm a block each, the rest shared.  Measured at
    // 256 x 8: 4.45 ms per call with one flight per block, 3.9 ms so; at 64 x 8: 2.76 and 2.67 ms.
    // Which flights share a block changes no bit of the result.  PE_GRAD_GROUP in the environment:
    // 1 gives every flight a block of its own in that kernel, 0 takes the one-flight kernel (the
    // same gradients to ~1e-6, its panel sums running over 4 warps instead of 3; it takes the
    // pipelined pass only in a small batch, as at 256 x 8 that gains it nothing).
    const char* group_env = getenv("PE_GRAD_GROUP");
    const int group_req = group_env ? atoi(group_env) : -1;
    a.group = store_forces && group_req != 0 ? grad_group_size(K) : 1;
    const bool small = nf <= 4 * e->nsm;
    if (store_forces && grad_long_pass(K) && (small || a.group > 1))
        a.n_long = std::min(nf, std::max(1, a.group > 1 && small ? e->nsm / 4 : e->nsm / 8));
    a.n_single = a.group > 1 ? (group_req == 1 ? nf : e->nsm) : 0;
    PE_CUDA(launch_grad(a, fa, e->nsm, e->g_fwd_bps, e->g_rev_grid, s, e->ev[2]));
    PE_CUDA(record_event(e->ev[3], s));
    // prepare (3), set-up, forward, order, reverse (two kernels with the pipelined pass), weights, genome
    e->last_launches = 3 + 6 + (a.n_long > 0 ? 1 : 0);
    e->prepared_pop = pop;
    e->timed = true;
    return PE_OK;
}

int pe_objective(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                 int max_steps, int precision, double* d_obj, double* d_dist, void* stream) {
    if (!e || !d_genomes) return fail(PE_EINVAL, "NULL engine or genomes");
    if (int rc = check_pop(pop)) return rc;
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (nseeds > kGradMaxSeeds) return fail(PE_EINVAL, "pe_objective takes at most %d seeds", kGradMaxSeeds);
    if (max_steps < 1 || max_steps > kMaxSteps) return fail(PE_EINVAL, "max_steps must be in 1..%d", kMaxSteps);
    if (precision != 32 && precision != 64) return fail(PE_EINVAL, "precision must be 32 or 64 (got %d)", precision);
    if ((long long)pop * nseeds > (1LL << 30)) return fail(PE_EINVAL, "pop * nseeds too large");
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nf = (size_t)pop * nseeds;
    PE_CUDA(e->o_plane.ensure((size_t)pop * kObjPlaneStride));  // sized for FP64, FP32 uses half
    if (!d_dist) PE_CUDA(e->o_dist.ensure(nf));
    PE_CUDA(e->o_work.ensure(1));
    if (int rc = upload_seeds(e, h_seeds, nseeds, s)) return rc;
    ObjArgs a{};
    a.genomes = d_genomes;
    a.seeds = e->seeds.p;
    a.pop = pop;
    a.nseeds = nseeds;
    a.vary = vary;
    a.max_steps = max_steps;
    a.plane = e->o_plane.p;
    a.dist = d_dist ? d_dist : e->o_dist.p;
    a.obj = d_obj;
    a.work = e->o_work.p;
    PE_CUDA(record_event(e->ev[0], s));
    PE_CUDA(launch_objective(a, precision, e->nsm, s));
    PE_CUDA(record_event(e->ev[1], s));
    PE_CUDA(record_event(e->ev[2], s));
    PE_CUDA(record_event(e->ev[3], s));
    e->last_launches = 2 + (d_obj ? 1 : 0);
    e->timed = true;
    return PE_OK;
}

int pe_robust_scores(const float* d_samples, int pop, int nseeds, float* d_scores, void* stream) {
    if (!d_samples || !d_scores) return fail(PE_EINVAL, "NULL samples or scores");
    if (pop < 0 || nseeds <= 0 || nseeds > 4096) return fail(PE_EINVAL, "need pop >= 0 and 1 <= nseeds <= 4096");
    PE_CUDA(launch_scores(d_samples, pop, nseeds, d_scores, (cudaStream_t)stream));
    return PE_OK;
}

int pe_plane_table(pe_engine* e, int pop, float* d_mp, int* d_nt, int* d_off, float* d_ext, float* d_pc,
                   float* d_pn, int* h_total_panels, void* stream) {
    if (!e) return fail(PE_EINVAL, "NULL engine");
    if (pop <= 0 || pop > e->prepared_pop) return fail(PE_EINVAL, "pop %d exceeds the prepared %d", pop, e->prepared_pop);
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int total = 0;
    PE_CUDA(cudaMemcpyAsync(&total, e->total.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PE_CUDA(cudaStreamSynchronize(s));
    if (pop < e->prepared_pop) {  // panels of the first pop planes
        int off_next = 0;
        PE_CUDA(cudaMemcpy(&off_next, e->off.p + pop, sizeof(int), cudaMemcpyDeviceToHost));
        total = off_next;
    }
    if (h_total_panels) *h_total_panels = total;
    if (d_mp) PE_CUDA(cudaMemcpyAsync(d_mp, e->mp.p, sizeof(float) * kMpN * pop, cudaMemcpyDeviceToDevice, s));
    if (d_nt) PE_CUDA(cudaMemcpyAsync(d_nt, e->nt.p, sizeof(int) * pop, cudaMemcpyDeviceToDevice, s));
    if (d_off) PE_CUDA(cudaMemcpyAsync(d_off, e->off.p, sizeof(int) * pop, cudaMemcpyDeviceToDevice, s));
    if (d_ext) PE_CUDA(cudaMemcpyAsync(d_ext, e->ext.p, sizeof(float4) * pop, cudaMemcpyDeviceToDevice, s));
    if (d_pc) PE_CUDA(cudaMemcpyAsync(d_pc, e->pc.p, sizeof(float4) * total, cudaMemcpyDeviceToDevice, s));
    if (d_pn) PE_CUDA(cudaMemcpyAsync(d_pn, e->pn.p, sizeof(float4) * total, cudaMemcpyDeviceToDevice, s));
    return PE_OK;
}

int pe_plane_info(pe_engine* e, int p, float* h_mp, float* h_ext, int* h_nt) {
    if (!e) return fail(PE_EINVAL, "NULL engine");
    if (p < 0 || p >= e->prepared_pop) return fail(PE_EINVAL, "plane %d outside the prepared %d", p, e->prepared_pop);
    if (int rc = ensure_device(e)) return rc;
    PE_CUDA(cudaDeviceSynchronize());
    if (h_mp) PE_CUDA(cudaMemcpy(h_mp, e->mp.p + (size_t)p * kMpN, sizeof(float) * kMpN, cudaMemcpyDeviceToHost));
    if (h_ext) PE_CUDA(cudaMemcpy(h_ext, e->ext.p + p, sizeof(float4), cudaMemcpyDeviceToHost));
    if (h_nt) PE_CUDA(cudaMemcpy(h_nt, e->nt.p + p, sizeof(int), cudaMemcpyDeviceToHost));
    return PE_OK;
}

int pe_last_timing(pe_engine* e, float* ms, int* launches) {
    if (!e || !ms) return fail(PE_EINVAL, "NULL argument");
    if (!e->timed) return fail(PE_EINVAL, "no evaluation has run on this engine");
    if (int rc = ensure_device(e)) return rc;
    PE_CUDA(cudaEventSynchronize(e->ev[3]));
    PE_CUDA(cudaEventElapsedTime(&ms[0], e->ev[0], e->ev[1]));
    PE_CUDA(cudaEventElapsedTime(&ms[1], e->ev[1], e->ev[2]));
    PE_CUDA(cudaEventElapsedTime(&ms[2], e->ev[2], e->ev[3]));
    if (launches) *launches = e->last_launches;
    return PE_OK;
}

int pe_autotune(pe_engine* e, const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                int max_steps, pe_config* best) {
    if (!e || !d_genomes) return fail(PE_EINVAL, "NULL engine or genomes");
    if (int rc = check_pop(pop)) return rc;
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (int rc = ensure_device(e)) return rc;
    // a sample big enough to fill the GPU several times over, small enough to time quickly
    const int want_flights = 256 * 1024;
    int sample = std::max(1, std::min(pop, (want_flights + nseeds - 1) / nseeds));
    const pe_config keep = e->cfg;
    const int lanes_opts[2] = {32, 16};
    const int warps_opts[4] = {1, 2, 4, 8};
    const int chunk_opts[2] = {600, 7200};
    float best_ms = 1e30f;
    pe_config best_cfg = keep;
    struct Ev {  // released on every return path
        cudaEvent_t e = nullptr;
        ~Ev() { if (e) cudaEventDestroy(e); }
    } t0, t1;
    PE_CUDA(cudaEventCreate(&t0.e));
    PE_CUDA(cudaEventCreate(&t1.e));
    int rc = PE_OK;
    for (int cap = 0; cap < 4 && rc == PE_OK; cap++)
    for (int li = 0; li < 2 && rc == PE_OK; li++)
        for (int wi = 0; wi < 4 && rc == PE_OK; wi++)
            for (int ci = 0; ci < 2 && rc == PE_OK; ci++) {
                pe_config c = keep;
                c.lanes = lanes_opts[li]; c.warps = warps_opts[wi]; c.chunk = chunk_opts[ci];
                c.blocks = 0; c.use_graph = 0; c.reg_cap = cap;
                if (!valid_config(c)) continue;
                e->cfg = c;
                if (blocks_for(e, c) <= 0) continue;
                float ms = 0;
                for (int rep = 0; rep < 2 && rc == PE_OK; rep++) {  // first run warms up
                    cudaEventRecord(t0.e, nullptr);
                    rc = pe_eval_batch(e, d_genomes, sample, h_seeds, nseeds, vary, max_steps, nullptr, nullptr,
                                       nullptr, nullptr);
                    cudaEventRecord(t1.e, nullptr);
                    if (rc == PE_OK && (cudaEventSynchronize(t1.e) != cudaSuccess ||
                                        cudaEventElapsedTime(&ms, t0.e, t1.e) != cudaSuccess)) {
                        (void)cudaGetLastError();
                        rc = fail(PE_ECUDA, "autotune: timing a candidate shape failed");
                    }
                }
                if (rc == PE_OK && ms < best_ms) { best_ms = ms; best_cfg = c; }
            }
    best_cfg.use_graph = keep.use_graph;
    e->cfg = rc == PE_OK ? best_cfg : keep;
    if (best) *best = e->cfg;
    return rc;
}

int pe_debug_release(pe_engine* e, int pop, const int* h_seeds, int nseeds, int vary, float* d_state_out,
                     void* stream) {
    if (!e || !d_state_out) return fail(PE_EINVAL, "NULL argument");
    if (pop <= 0 || pop > e->prepared_pop) return fail(PE_EINVAL, "pop %d exceeds the prepared %d", pop, e->prepared_pop);
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = upload_seeds(e, h_seeds, nseeds, s)) return rc;
    FlightArgs a = flight_args(e, pop, nseeds, vary, kMaxSteps, nullptr, nullptr);
    PE_CUDA(launch_debug_release(a, (FlightState*)d_state_out, s));
    return PE_OK;
}

int pe_debug_step(pe_engine* e, int pop, const int* h_seeds, int nseeds, int vary, int max_steps,
                  const float* d_state_in, float* d_state_out, float* d_FT, int* d_done, float* d_fit, int step,
                  int lanes, void* stream) {
    if (!e || !d_state_in || !d_state_out || !d_FT || !d_done || !d_fit) return fail(PE_EINVAL, "NULL argument");
    if (pop <= 0 || pop > e->prepared_pop) return fail(PE_EINVAL, "pop %d exceeds the prepared %d", pop, e->prepared_pop);
    if (lanes != 16 && lanes != 32) return fail(PE_EINVAL, "lanes must be 16 or 32");
    if (e->cfg.formulation == 0 && lanes != 32) return fail(PE_EINVAL, "the reference arithmetic runs 32 lanes per flight");
    if (step < 0 || max_steps < 1 || max_steps > kMaxSteps) return fail(PE_EINVAL, "bad step/max_steps");
    if (int rc = check_seeds(h_seeds, nseeds)) return rc;
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = upload_seeds(e, h_seeds, nseeds, s)) return rc;
    FlightArgs a = flight_args(e, pop, nseeds, vary, max_steps, nullptr, nullptr);
    if (e->cfg.formulation)
        PE_CUDA(launch_debug_step_fast(a, (const FlightState*)d_state_in, (FlightState*)d_state_out, d_FT, d_done,
                                       d_fit, step, lanes, s));
    else
        PE_CUDA(launch_debug_step(a, (const FlightState*)d_state_in, (FlightState*)d_state_out, d_FT, d_done, d_fit,
                                  step, lanes, s));
    return PE_OK;
}

int pe_debug_station_mode(int ieee) {
    PE_CUDA(set_station_mode(ieee));
    return PE_OK;
}

int pe_debug_fail_evaluations(int after_calls) {
    g_eval_budget.store(after_calls < 0 ? -1 : after_calls);
    return PE_OK;
}

// ---------------------------------------------------------------- reference-compatible layer
struct pe_panelbuf {
    pe_engine* e;
    int cap;
};

int pe_panelbuf_alloc(int pop, void** out_pb) {
    if (!out_pb) return fail(PE_EINVAL, "out_pb is NULL");
    *out_pb = nullptr;
    if (int rc = check_pop(pop)) return rc;
    int dev = 0;
    PE_CUDA(cudaGetDevice(&dev));
    pe_engine* e = nullptr;
    if (int rc = pe_engine_create(dev, &e)) return rc;
    if (int rc = engine_reserve(e, pop, pop)) { pe_engine_destroy(e); return rc; }
    pe_panelbuf* pb = new pe_panelbuf{e, pop};
    *out_pb = pb;
    return PE_OK;
}

int pe_panelbuf_free(void* pbv) {
    if (!pbv) return PE_OK;
    pe_panelbuf* pb = (pe_panelbuf*)pbv;
    pe_engine_destroy(pb->e);
    delete pb;
    return PE_OK;
}

int pe_prepare(const float* d_genomes, void* pbv, int pop, void* stream) {
    if (!pbv || !d_genomes) return fail(PE_EINVAL, "NULL panelbuf or genomes");
    pe_panelbuf* pb = (pe_panelbuf*)pbv;
    if (pop <= 0 || pop > pb->cap) return fail(PE_EINVAL, "pop %d outside 1..%d", pop, pb->cap);
    pe_engine* e = pb->e;
    if (int rc = ensure_device(e)) return rc;
    launch_prepare(prep_args(e, d_genomes, pop), e->total.p, (cudaStream_t)stream);
    PE_CUDA(cudaGetLastError());
    e->prepared_pop = pop;
    return PE_OK;
}

int pe_sim(void* pbv, int pop, int seed, float* d_fitness, float* d_rec, int rec_every, int rec_cap,
           float launch_spread, int vary_scenarios, void* stream) {
    if (!pbv || !d_fitness) return fail(PE_EINVAL, "NULL panelbuf or fitness");
    pe_panelbuf* pb = (pe_panelbuf*)pbv;
    pe_engine* e = pb->e;
    if (pop <= 0 || pop > e->prepared_pop) return fail(PE_EINVAL, "pop %d exceeds the prepared %d", pop, e->prepared_pop);
    if (d_rec && (rec_every < 1 || rec_cap < 0))
        return fail(PE_EINVAL, "recording needs rec_every >= 1 and rec_cap >= 0 (got %d, %d)", rec_every, rec_cap);
    if (int rc = ensure_device(e)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = engine_reserve(e, pop, pop)) return rc;
    if (int rc = upload_seeds(e, &seed, 1, s)) return rc;
    if (d_rec || launch_spread > 0.0f) {
        // pose recording / launch grid: one launch of the default shape over the whole horizon
        FlightShape sh{16, 2, kMaxSteps, 0, 1, 0};
        FlightArgs a = flight_args(e, pop, 1, vary_scenarios ? 1 : 0, kMaxSteps, d_fitness, e->steps_tmp.p);
        a.step_begin = 0;
        a.step_end = kMaxSteps;
        a.work = e->counters.p;
        a.rec = d_rec;
        a.rec_every = d_rec ? rec_every : 1;
        a.rec_cap = d_rec ? rec_cap : 0;
        a.spread = launch_spread;
        int bps = flight_fast_blocks_per_sm(sh);
        PE_CUDA(cudaMemsetAsync(e->counters.p, 0, sizeof(int), s));
        PE_CUDA(launch_flight_fast(a, sh, (bps > 0 ? bps : 1) * e->nsm, s));
        PE_CUDA(cudaStreamSynchronize(s));
        return PE_OK;
    }
    int launches = 0;
    if (int rc = enqueue_fly(e, pop, 1, vary_scenarios ? 1 : 0, kMaxSteps, d_fitness, e->steps_tmp.p, s, &launches))
        return rc;
    PE_CUDA(cudaStreamSynchronize(s));
    return PE_OK;
}

}  // extern "C"
