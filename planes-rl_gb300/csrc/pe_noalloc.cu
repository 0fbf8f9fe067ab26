// pe_noalloc.cu -- pe_eval_batch_noalloc: the batched evaluation without any allocation.
//
// Who needs it: callers that cannot call cudaMalloc at the moment they evaluate, e.g. hosts
// whose device memory is entirely pre-reserved by their own pooling allocator (a cudaMalloc
// there fails or evicts their pool), or real-time loops whose latency budget forbids a trip
// through the driver's allocator and its implicit synchronization.  They pass genomes and output
// buffers they already own; every piece of working memory (plane table, packed panels, seeds,
// launch counters, and distances when the caller passes none) lives in the one file-scope device
// array below.
//
// Limits: at most kNaMaxPlanes genomes and kNaMaxFlights flights (pop x nseeds) per call; larger
// requests are rejected with PE_EINVAL.  The array (about 2.9 MB) is resident on every GPU that
// loads the library until the process exits.
//
// Sharing: every call on a device uses the same array and leaves its contents behind; each call
// clears the counters that must start at zero.  Calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the array and must be serialized by the caller.
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress while that device is current (the host-side name of a __device__ array
// is only a stand-in, not a device address), and keeps it for the life of the process; a
// cudaDeviceReset leaves that address stale, so do not reset a device this entry has used.
// Make that first call before any stream capture.
#include <stdio.h>

#include <mutex>

#include "../../include/planes_eval.h"
#include "pe_internal.cuh"

namespace pe {
namespace {

constexpr int kNaMaxPlanes = 256;
constexpr int kNaMaxFlights = 4096;
constexpr int kNaMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// byte offsets of the regions inside the array
constexpr size_t kOffNt = 0;
constexpr size_t kOffOff = kOffNt + align256(sizeof(int) * kNaMaxPlanes);
constexpr size_t kOffTopo = kOffOff + align256(sizeof(int) * kNaMaxPlanes);
constexpr size_t kOffBlock = kOffTopo + align256(sizeof(int) * kNaMaxPlanes);
constexpr size_t kOffTotal = kOffBlock + align256(sizeof(int) * 4);
constexpr size_t kOffMp = kOffTotal + align256(sizeof(int));
constexpr size_t kOffExt = kOffMp + align256(sizeof(float) * kMpN * kNaMaxPlanes);
constexpr size_t kOffPc = kOffExt + align256(sizeof(float4) * kNaMaxPlanes);
constexpr size_t kOffPn = kOffPc + align256(sizeof(float4) * kNtMax * kNaMaxPlanes);
constexpr size_t kOffSeeds = kOffPn + align256(sizeof(float4) * kNtMax * kNaMaxPlanes);
constexpr size_t kOffCounters = kOffSeeds + align256(sizeof(int) * kNaMaxFlights);
constexpr size_t kOffDist = kOffCounters + align256(sizeof(int) * 4);
constexpr size_t kOffSteps = kOffDist + align256(sizeof(float) * kNaMaxFlights);
constexpr size_t kNaBytes = kOffSteps + align256(sizeof(int) * kNaMaxFlights);

// The working memory of pe_eval_batch_noalloc.  Host code must not use this name as a device
// address: it reaches the array only through the pointer cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

std::mutex g_mu;
unsigned char* g_base[kNaMaxDevices] = {};
int g_grid[kNaMaxDevices] = {};

// The fixed execution shape of this entry point: body-frame formulation, 16 lanes per flight,
// one-warp blocks (register budget 3), the whole flight in one launch (no saved state, no
// airborne lists).
constexpr FlightShape kShape{16, 1, kMaxSteps, 0, 1, 3};

}  // namespace
}  // namespace pe

using namespace pe;

namespace {
// A CUDA failure of this entry: cleared from the runtime's last-error slot (it is reported here)
// and described for pe_last_error().
int na_fail(const char* what) {
    (void)cudaGetLastError();
    pe::set_last_error(what);
    return PE_ECUDA;
}
}  // namespace

extern "C" int pe_eval_batch_noalloc(const float* d_genomes, int pop, const int* h_seeds, int nseeds, int vary,
                                     int max_steps, float* d_dist, int* d_steps, float* d_scores, void* stream) {
    if (!d_genomes || !h_seeds) {
        set_last_error("pe_eval_batch_noalloc: NULL genomes or seeds");
        return PE_EINVAL;
    }
    if (pop <= 0 || nseeds <= 0 || max_steps < 1 || max_steps > kMaxSteps) {
        set_last_error("pe_eval_batch_noalloc: need pop > 0, nseeds > 0 and 1 <= max_steps <= 7200");
        return PE_EINVAL;
    }
    if (pop > kNaMaxPlanes || (long long)pop * nseeds > kNaMaxFlights) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "pe_eval_batch_noalloc: %d genomes x %d scenarios exceeds its static working memory "
                 "(at most %d genomes and %d flights per call)",
                 pop, nseeds, kNaMaxPlanes, kNaMaxFlights);
        set_last_error(msg);
        return PE_EINVAL;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return na_fail("pe_eval_batch_noalloc: no usable current device");
    unsigned char* base = nullptr;
    int grid = 0;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_base[dev]) {  // once per device, with that device current
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return na_fail("pe_eval_batch_noalloc: static scratch not found on this device");
            int nsm = 0;
            if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return na_fail("pe_eval_batch_noalloc: device attribute query failed");
            const int bps = flight_fast_blocks_per_sm(kShape);
            if (bps <= 0) return na_fail("pe_eval_batch_noalloc: flight kernel cannot reside on this device");
            g_grid[dev] = bps * nsm;
            g_base[dev] = (unsigned char*)p;
        }
        base = g_base[dev];
        grid = g_grid[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    int* counters = (int*)(base + kOffCounters);
    float* dist = d_dist ? d_dist : (float*)(base + kOffDist);
    int* steps = d_steps ? d_steps : (int*)(base + kOffSteps);
    int* seeds = (int*)(base + kOffSeeds);
    // the seeds, then the counters that must start at zero (the array keeps the last call's values)
    if (cudaMemcpyAsync(seeds, h_seeds, sizeof(int) * nseeds, cudaMemcpyHostToDevice, s) != cudaSuccess) return na_fail("pe_eval_batch_noalloc: seed upload failed");
    if (cudaMemsetAsync(counters, 0, sizeof(int) * 4, s) != cudaSuccess) return na_fail("pe_eval_batch_noalloc: counter reset failed");

    PrepArgs pa;
    pa.genomes = d_genomes;
    pa.pop = pop;
    pa.nt_topo = (int*)(base + kOffTopo);
    pa.block_sum = (int*)(base + kOffBlock);
    pa.pt.nt = (int*)(base + kOffNt);
    pa.pt.off = (int*)(base + kOffOff);
    pa.pt.mp = (float*)(base + kOffMp);
    pa.pt.ext = (float4*)(base + kOffExt);
    pa.pc = (float4*)(base + kOffPc);
    pa.pn = (float4*)(base + kOffPn);
    launch_prepare(pa, (int*)(base + kOffTotal), s);
    if (cudaGetLastError() != cudaSuccess) return na_fail("pe_eval_batch_noalloc: prepare launch failed");

    FlightArgs fa{};
    fa.pc = pa.pc;
    fa.pn = pa.pn;
    fa.plane_nt = pa.pt.nt;
    fa.plane_off = pa.pt.off;
    fa.plane_mp = pa.pt.mp;
    fa.seeds = seeds;
    fa.nseeds = nseeds;
    fa.vary = vary ? 1 : 0;
    fa.max_steps = max_steps;
    fa.n_flights = pop * nseeds;
    fa.step_begin = 0;
    fa.step_end = max_steps;  // every flight ends inside this launch: no state is saved
    fa.active_in = nullptr;
    fa.n_active_in = counters + 1;
    fa.active_out = nullptr;
    fa.n_active_out = counters + 2;
    fa.work = counters;
    fa.state = nullptr;
    fa.dist = dist;
    fa.steps = steps;
    if (launch_flight_fast(fa, kShape, grid, s) != cudaSuccess) return na_fail("pe_eval_batch_noalloc: flight launch failed");
    if (d_scores && launch_scores(dist, pop, nseeds, d_scores, s) != cudaSuccess) return na_fail("pe_eval_batch_noalloc: scores launch failed");
    return PE_OK;
}
