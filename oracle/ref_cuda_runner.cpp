// ref_cuda_runner.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CUDA kernels (k_prepare, k_sim of src/sim.cu, compiled by
// oracle/build.py into oracle/_ref/ref_sim.ptx with the reference's flags) on a GPU through the
// CUDA driver API, driving them the way the reference's host code does:
//   gpu_prepare  = k_prepare<<<pop, 64>>>                                  (src/sim.cu:214-218)
//   gpu_sim      = 12 x { k_sim<<<pop, 128>>>(..., step0, 600); sync }     (src/sim.cu:238-248)
// It records the reference build's outputs (golden vectors for tests/golden) and its wall time.
//
//   ref_cuda_runner <ptx> eval    <genomes.bin> <pop> <vary> <out_dir> <seed>...
//       prepare once, then gpu_sim per seed (the GA's training loop, src/sim.cu:433-438);
//       writes fitness.bin [pop][nseeds], mp.bin [pop][20], nt.bin [pop], pc.bin/pn.bin
//       [min(pop,256)][900][4], timing.txt
//   ref_cuda_runner <ptx> step    <genomes.bin> <pop> <vary> <seed> <states.bin> <step0> <nsteps> <out_dir>
//       prepare, load PlaneState [pop] (15 floats), one k_sim launch (step0, nsteps) that resumes
//       from them (its clock restarts at step0 * SIM_DT); writes states.bin, fitness.bin
//   ref_cuda_runner <ptx> release <genomes.bin> <pop> <vary> <seed> <out_dir>
//       prepare and one k_sim launch with step0 = 0, nsteps = 0: the release states
//   ref_cuda_runner <ptx> record  <genomes.bin> <pop> <vary> <seed> <rec_every> <rec_cap> <spread> <out_dir>
//       prepare and gpu_sim with pose recording and the launch grid (src/sim.cu:238-248 with d_rec,
//       as render.cu drives it); the record buffer starts as NaN; writes rec.bin
//       [pop][rec_cap][8] and fitness.bin
//   ref_cuda_runner <ptx> traj    <genomes.bin> <pop> <vary> <seed> <out_dir> <k>...
//       for each k: prepare, then the launches gpu_sim makes up to step k (600-step chunks, the
//       last one cut at k; the first one releases), then one resumed launch (step0 = k,
//       nsteps = 1); writes in_<k>.bin (states at k) and out_<k>.bin (states at k + 1), [pop][15]
//   ref_cuda_runner <ptx> gen     <genomes.bin> <pop> <vary> <out_dir> <reps> <holdout> <holdout_base>
//                                 <topk> <seed>...
//       one generation of run_ga per rep (src/sim.cu:431-456), host to host: genomes H2D, prepare,
//       gpu_sim + D2H per training seed, the tail-aware score on the host, the top `topk`, each
//       flown on `holdout` copies with gpu_sim(holdout_base, vary 1); the first rep is a warm-up.
//       Writes fitness.bin [pop][nseeds], scores.bin [pop], top.bin [topk] int, holdout.bin
//       [topk][holdout] of the last rep, and timing.txt (seconds of every timed rep)
#include <cuda.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define CK(x)                                                                                   \
    do {                                                                                        \
        CUresult r_ = (x);                                                                      \
        if (r_ != CUDA_SUCCESS) {                                                               \
            const char* s_ = nullptr;                                                           \
            cuGetErrorString(r_, &s_);                                                          \
            fprintf(stderr, "CUDA driver error %s at %s:%d: %s\n", s_ ? s_ : "?", __FILE__, __LINE__, #x); \
            exit(2);                                                                            \
        }                                                                                       \
    } while (0)

static const int kMaxT = 900;       // MAX_T of the reference
static const int kSimMax = 7200;    // SIM_MAX_STEPS
static const int kChunk = 600;      // gpu_sim's CHUNK

struct PanelBufDev {  // layout of the reference's PanelBuf (src/sim.cu:15-21): five pointers
    CUdeviceptr pc, pn, mp, nt, st;
};

static std::vector<char> read_file(const std::string& p) {
    FILE* f = fopen(p.c_str(), "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", p.c_str()); exit(2); }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> b(n + 1, 0);
    if (fread(b.data(), 1, n, f) != (size_t)n) { fprintf(stderr, "short read %s\n", p.c_str()); exit(2); }
    fclose(f);
    b.resize(n);
    return b;
}

static void write_file(const std::string& p, const void* d, size_t n) {
    FILE* f = fopen(p.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", p.c_str()); exit(2); }
    fwrite(d, 1, n, f);
    fclose(f);
}

struct Ref {
    CUmodule mod;
    CUfunction prep = nullptr, sim = nullptr;
    PanelBufDev pb{};
    int cap = 0;

    void load(const std::string& ptx_path) {
        std::vector<char> ptx = read_file(ptx_path);
        ptx.push_back(0);
        CK(cuModuleLoadData(&mod, ptx.data()));
        unsigned n = 0;
        CK(cuModuleGetFunctionCount(&n, mod));
        std::vector<CUfunction> fs(n);
        CK(cuModuleEnumerateFunctions(fs.data(), n, mod));
        for (CUfunction f : fs) {
            const char* name = nullptr;
            CK(cuFuncGetName(&name, f));
            if (strstr(name, "k_prepare")) prep = f;
            if (strstr(name, "k_sim")) sim = f;
        }
        if (!prep || !sim) { fprintf(stderr, "kernels not found in %s\n", ptx_path.c_str()); exit(2); }
    }
    void alloc(int pop) {  // panelbuf_alloc, src/sim.cu:220-228
        cap = pop;
        CK(cuMemAlloc(&pb.pc, 16ull * pop * kMaxT));
        CK(cuMemAlloc(&pb.pn, 16ull * pop * kMaxT));
        CK(cuMemAlloc(&pb.mp, 80ull * pop));
        CK(cuMemAlloc(&pb.nt, 4ull * pop));
        CK(cuMemAlloc(&pb.st, 60ull * pop));
    }
    void prepare(CUdeviceptr gs, int pop) {
        void* args[] = {&gs, &pb, &pop};
        CK(cuLaunchKernel(prep, pop, 1, 1, 64, 1, 1, 0, nullptr, args, nullptr));
    }
    void sim_launch(int pop, int seed, CUdeviceptr fit, int vary, int step0, int nsteps, CUdeviceptr rec = 0,
                    int rec_every = 1, int rec_cap = 0, float spread = 0.0f) {
        CUdeviceptr st = pb.st;
        void* args[] = {&pb, &pop, &seed, &fit, &rec, &rec_every, &rec_cap, &spread, &vary, &st, &step0, &nsteps};
        CK(cuLaunchKernel(sim, pop, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr));
    }
    void gpu_sim(int pop, int seed, CUdeviceptr fit, int vary, CUdeviceptr rec = 0, int rec_every = 1,
                 int rec_cap = 0, float spread = 0.0f) {  // src/sim.cu:238-248
        for (int s0 = 0; s0 < kSimMax; s0 += kChunk) {
            sim_launch(pop, seed, fit, vary, s0, kChunk, rec, rec_every, rec_cap, spread);
            CK(cuCtxSynchronize());
        }
    }
};

// The tail-aware score of src/sim.cu:340-357 (float, the reference's order of operations).
static void robust_scores(const std::vector<float>& samples, int pop, int nseeds, std::vector<float>& scores) {
    std::vector<float> row(nseeds);
    const int tail_n = (nseeds + 3) / 4;
    scores.resize(pop);
    for (int i = 0; i < pop; i++) {
        float mean = 0;
        for (int s = 0; s < nseeds; s++) {
            row[s] = samples[(size_t)i * nseeds + s];
            mean += row[s] / nseeds;
        }
        std::sort(row.begin(), row.end());
        float cvar = 0;
        for (int s = 0; s < tail_n; s++) cvar += row[s] / tail_n;
        scores[i] = 0.65f * mean + 0.25f * cvar + 0.10f * row[0];
    }
}

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: see header\n"); return 2; }
    std::string ptx = argv[1], mode = argv[2];
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    Ref ref;
    ref.load(ptx);

    std::vector<char> graw = read_file(argv[3]);
    int pop = atoi(argv[4]);
    int vary = atoi(argv[5]);
    if ((size_t)pop * 140 > graw.size()) { fprintf(stderr, "genome file too short\n"); return 2; }
    CUdeviceptr d_gs, d_fit;
    CK(cuMemAlloc(&d_gs, 140ull * pop));
    ref.alloc(pop);

    if (mode == "eval") {
        std::string out = argv[6];
        std::vector<int> seeds;
        for (int i = 7; i < argc; i++) seeds.push_back(atoi(argv[i]));
        int S = (int)seeds.size();
        CK(cuMemAlloc(&d_fit, 4ull * pop));
        std::vector<float> fit(pop), samples((size_t)pop * S);
        CK(cuCtxSynchronize());
        auto t0 = std::chrono::steady_clock::now();
        CK(cuMemcpyHtoD(d_gs, graw.data(), 140ull * pop));
        ref.prepare(d_gs, pop);
        CK(cuCtxSynchronize());
        auto t1 = std::chrono::steady_clock::now();
        for (int s = 0; s < S; s++) {
            ref.gpu_sim(pop, seeds[s], d_fit, vary);
            CK(cuMemcpyDtoH(fit.data(), d_fit, 4ull * pop));
            for (int i = 0; i < pop; i++) samples[(size_t)i * S + s] = fit[i];
        }
        auto t2 = std::chrono::steady_clock::now();
        double prep_s = std::chrono::duration<double>(t1 - t0).count();
        double sim_s = std::chrono::duration<double>(t2 - t1).count();
        write_file(out + "/fitness.bin", samples.data(), samples.size() * 4);
        std::vector<float> mp((size_t)pop * 20);
        std::vector<int> nt(pop);
        CK(cuMemcpyDtoH(mp.data(), ref.pb.mp, 80ull * pop));
        CK(cuMemcpyDtoH(nt.data(), ref.pb.nt, 4ull * pop));
        write_file(out + "/mp.bin", mp.data(), mp.size() * 4);
        write_file(out + "/nt.bin", nt.data(), nt.size() * 4);
        int kp = pop < 256 ? pop : 256;
        std::vector<float> pc((size_t)kp * kMaxT * 4), pn((size_t)kp * kMaxT * 4);
        CK(cuMemcpyDtoH(pc.data(), ref.pb.pc, pc.size() * 4));
        CK(cuMemcpyDtoH(pn.data(), ref.pb.pn, pn.size() * 4));
        write_file(out + "/pc.bin", pc.data(), pc.size() * 4);
        write_file(out + "/pn.bin", pn.data(), pn.size() * 4);
        FILE* f = fopen((out + "/timing.txt").c_str(), "w");
        fprintf(f, "pop %d nseeds %d vary %d prepare_s %.6f sim_s %.6f launches %d\n", pop, S, vary, prep_s,
                sim_s, 1 + S * (kSimMax / kChunk));
        fclose(f);
        printf("ref eval pop %d nseeds %d: prepare %.3f s, flights %.3f s\n", pop, S, prep_s, sim_s);
    } else if (mode == "step" || mode == "release") {
        int seed = atoi(argv[6]);
        CK(cuMemAlloc(&d_fit, 4ull * pop));
        CK(cuMemsetD8(d_fit, 0, 4ull * pop));
        CK(cuMemcpyHtoD(d_gs, graw.data(), 140ull * pop));
        ref.prepare(d_gs, pop);
        std::string out;
        if (mode == "step") {
            std::vector<char> sraw = read_file(argv[7]);
            if (sraw.size() < 60ull * pop) { fprintf(stderr, "state file too short\n"); return 2; }
            int step0 = atoi(argv[8]), nsteps = atoi(argv[9]);
            out = argv[10];
            if (step0 < 1) { fprintf(stderr, "step0 must be >= 1 to resume from a state\n"); return 2; }
            CK(cuMemcpyHtoD(ref.pb.st, sraw.data(), 60ull * pop));
            ref.sim_launch(pop, seed, d_fit, vary, step0, nsteps);
        } else {
            out = argv[7];
            ref.sim_launch(pop, seed, d_fit, vary, 0, 0);
        }
        CK(cuCtxSynchronize());
        std::vector<float> st((size_t)pop * 15), fit(pop);
        CK(cuMemcpyDtoH(st.data(), ref.pb.st, 60ull * pop));
        CK(cuMemcpyDtoH(fit.data(), d_fit, 4ull * pop));
        write_file(out + "/states.bin", st.data(), st.size() * 4);
        write_file(out + "/fitness.bin", fit.data(), fit.size() * 4);
    } else if (mode == "record") {
        if (argc < 11) { fprintf(stderr, "record: <seed> <rec_every> <rec_cap> <spread> <out_dir>\n"); return 2; }
        const int seed = atoi(argv[6]), rec_every = atoi(argv[7]), rec_cap = atoi(argv[8]);
        const float spread = (float)atof(argv[9]);
        const std::string out = argv[10];
        if (rec_every < 1 || rec_cap < 1) { fprintf(stderr, "record needs rec_every >= 1, rec_cap >= 1\n"); return 2; }
        CUdeviceptr d_rec;
        const size_t nrec = (size_t)pop * rec_cap * 8;
        CK(cuMemAlloc(&d_fit, 4ull * pop));
        CK(cuMemAlloc(&d_rec, 4 * nrec));
        CK(cuMemsetD32(d_rec, 0x7fc00000u, nrec));  // NaN: slots the kernel never writes stay NaN
        CK(cuMemcpyHtoD(d_gs, graw.data(), 140ull * pop));
        ref.prepare(d_gs, pop);
        ref.gpu_sim(pop, seed, d_fit, vary, d_rec, rec_every, rec_cap, spread);
        std::vector<float> rec(nrec), fit(pop);
        CK(cuMemcpyDtoH(rec.data(), d_rec, 4 * nrec));
        CK(cuMemcpyDtoH(fit.data(), d_fit, 4ull * pop));
        write_file(out + "/rec.bin", rec.data(), rec.size() * 4);
        write_file(out + "/fitness.bin", fit.data(), fit.size() * 4);
    } else if (mode == "traj") {
        if (argc < 9) { fprintf(stderr, "traj: <seed> <out_dir> <k>...\n"); return 2; }
        const int seed = atoi(argv[6]);
        const std::string out = argv[7];
        CK(cuMemAlloc(&d_fit, 4ull * pop));
        CK(cuMemcpyHtoD(d_gs, graw.data(), 140ull * pop));
        std::vector<float> st((size_t)pop * 15);
        for (int a = 8; a < argc; a++) {
            const int k = atoi(argv[a]);
            if (k < 1 || k >= kSimMax) { fprintf(stderr, "traj: k must be in 1..%d\n", kSimMax - 1); return 2; }
            CK(cuMemsetD8(d_fit, 0, 4ull * pop));
            ref.prepare(d_gs, pop);
            for (int s0 = 0; s0 < k; s0 += kChunk) ref.sim_launch(pop, seed, d_fit, vary, s0, std::min(kChunk, k - s0));
            CK(cuCtxSynchronize());
            CK(cuMemcpyDtoH(st.data(), ref.pb.st, 60ull * pop));
            write_file(out + "/in_" + std::to_string(k) + ".bin", st.data(), st.size() * 4);
            ref.sim_launch(pop, seed, d_fit, vary, k, 1);
            CK(cuCtxSynchronize());
            CK(cuMemcpyDtoH(st.data(), ref.pb.st, 60ull * pop));
            write_file(out + "/out_" + std::to_string(k) + ".bin", st.data(), st.size() * 4);
        }
    } else if (mode == "gen") {
        if (argc < 12) { fprintf(stderr, "gen: <out_dir> <reps> <holdout> <holdout_base> <topk> <seed>...\n"); return 2; }
        const std::string out = argv[6];
        const int reps = atoi(argv[7]), H = atoi(argv[8]), hbase = atoi(argv[9]), K = atoi(argv[10]);
        std::vector<int> seeds;
        for (int i = 11; i < argc; i++) seeds.push_back(atoi(argv[i]));
        const int S = (int)seeds.size();
        if (reps < 1 || H < 1 || K < 1 || K > pop) { fprintf(stderr, "gen: need reps, holdout >= 1, 1 <= topk <= pop\n"); return 2; }
        CK(cuMemAlloc(&d_fit, 4ull * pop));
        Ref val;  // the holdout's own panel buffers (run_ga's val_pb), same module
        val.mod = ref.mod; val.prep = ref.prep; val.sim = ref.sim;
        val.alloc(H);
        CUdeviceptr d_val_gs, d_val_fit;
        CK(cuMemAlloc(&d_val_gs, 140ull * H));
        CK(cuMemAlloc(&d_val_fit, 4ull * H));
        std::vector<float> fit(pop), samples((size_t)pop * S), scores, hold((size_t)K * H);
        std::vector<char> copies(140ull * H);
        std::vector<int> idx(pop);
        std::vector<double> secs;
        for (int r = 0; r <= reps; r++) {
            CK(cuCtxSynchronize());
            auto t0 = std::chrono::steady_clock::now();
            CK(cuMemcpyHtoD(d_gs, graw.data(), 140ull * pop));
            ref.prepare(d_gs, pop);
            for (int s = 0; s < S; s++) {
                ref.gpu_sim(pop, seeds[s], d_fit, vary);
                CK(cuMemcpyDtoH(fit.data(), d_fit, 4ull * pop));
                for (int i = 0; i < pop; i++) samples[(size_t)i * S + s] = fit[i];
            }
            robust_scores(samples, pop, S, scores);
            for (int i = 0; i < pop; i++) idx[i] = i;
            std::partial_sort(idx.begin(), idx.begin() + K, idx.end(), [&](int a, int b) {
                return scores[a] > scores[b] || (scores[a] == scores[b] && a < b);
            });
            for (int c = 0; c < K; c++) {
                for (int i = 0; i < H; i++) memcpy(&copies[140ull * i], &graw[140ull * idx[c]], 140);
                CK(cuMemcpyHtoD(d_val_gs, copies.data(), 140ull * H));
                val.prepare(d_val_gs, H);
                val.gpu_sim(H, hbase, d_val_fit, 1);
                CK(cuMemcpyDtoH(&hold[(size_t)c * H], d_val_fit, 4ull * H));
            }
            auto t1 = std::chrono::steady_clock::now();
            if (r > 0) secs.push_back(std::chrono::duration<double>(t1 - t0).count());
        }
        write_file(out + "/fitness.bin", samples.data(), samples.size() * 4);
        write_file(out + "/scores.bin", scores.data(), scores.size() * 4);
        write_file(out + "/top.bin", idx.data(), 4ull * K);
        write_file(out + "/holdout.bin", hold.data(), hold.size() * 4);
        FILE* f = fopen((out + "/timing.txt").c_str(), "w");
        if (!f) { fprintf(stderr, "cannot write timing.txt\n"); return 2; }
        fprintf(f, "pop %d nseeds %d holdout %d topk %d reps %d seconds", pop, S, H, K, reps);
        for (double x : secs) fprintf(f, " %.6f", x);
        fprintf(f, "\n");
        fclose(f);
        printf("ref generation pop %d x %d + top-%d x %d holdout:", pop, S, K, H);
        for (double x : secs) printf(" %.3f s", x);
        printf("\n");
    } else {
        fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    return 0;
}
