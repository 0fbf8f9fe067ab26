// pe_drivers.cpp -- the reference's evaluate / select-best / evolve drivers (src/sim.cu:250-520)
// on top of the batched engine.  Seeding, file formats, CSV columns and printed summaries follow
// the reference; the evaluation itself runs as one batched call per population instead of one
// 12-launch gpu_sim per scenario seed.
//
//   evaluate_design: one genome x N scenarios, env_seed = base + i * 7919 (src/sim.cu:258-312)
//   select_finalist: C candidates x N scenarios in a single batch (src/sim.cu:359-391)
//   run_ga:          the GA of src/sim.cu:393-520 with the same std::mt19937(42) stream, so the
//                    same fitness values give the same populations and files
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "planes_eval.h"

namespace pe {
void set_last_error(const char* msg);  // pe_api.cu
}

namespace {

// Host scenario draw for the telemetry CSV (src/common.h:368-421), in the host arithmetic the
// reference's CSV is written with.
uint32_t mix_bits(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
float su01(int seed, int lane) {
    return (mix_bits((uint32_t)seed * 0x9e3779b9u + (uint32_t)lane * 0x85ebca6bu) >> 8) * (1.0f / 16777216.0f);
}
float ssg(int seed, int lane) { return su01(seed, lane) * 2.0f - 1.0f; }

struct Scen {
    float speed, pitch, yaw, roll, height, roll_rate, pitch_rate, yaw_rate, air_rho, skin_cf, gust, base_x,
        base_y, force_pitch, force_yaw, grip_x, grip_y, grip_z, material_scale, infill_ratio, bias_x, bias_y,
        bias_z, warp_pitch, warp_roll;
};

Scen scenario(int seed) {
    Scen d;
    d.speed = 9.2f + 2.0f * ssg(seed, 0);
    d.pitch = 0.10f + 0.20f * ssg(seed, 1);
    d.yaw = 0.12f * ssg(seed, 2);
    d.roll = 0.16f * ssg(seed, 3);
    d.height = 1.75f + 0.35f * ssg(seed, 4);
    d.roll_rate = 1.8f * ssg(seed, 5);
    d.pitch_rate = 1.2f * ssg(seed, 6);
    d.yaw_rate = 1.5f * ssg(seed, 7);
    d.air_rho = 1.225f * (0.88f + 0.22f * su01(seed, 8));
    d.skin_cf = 0.02f * (0.75f + 0.55f * su01(seed, 9));
    d.gust = 0.45f + 1.10f * (0.5f + 0.5f * sinf(seed * 1.61803f));
    float phase = (float)((int)((uint32_t)seed * 37u) % 97);
    d.base_x = -0.25f + 1.15f * sinf(phase * 0.71f);
    d.base_y = 1.00f * sinf(phase * 1.13f);
    d.force_pitch = 0.075f * ssg(seed, 10);
    d.force_yaw = 0.060f * ssg(seed, 11);
    d.grip_x = 0.018f * ssg(seed, 12);
    d.grip_y = 0.022f * ssg(seed, 13);
    d.grip_z = 0.010f * ssg(seed, 14);
    d.material_scale = 0.88f + 0.24f * su01(seed, 15);
    d.infill_ratio = 0.06f + 0.34f * su01(seed, 16);
    d.bias_x = 0.018f * ssg(seed, 17);
    d.bias_y = 0.010f * ssg(seed, 18);
    d.bias_z = 0.006f * ssg(seed, 19);
    d.skin_cf *= 0.90f + 0.25f * su01(seed, 20);
    d.warp_pitch = 0.025f * ssg(seed, 21);
    d.warp_roll = 0.035f * ssg(seed, 22);
    return d;
}

void mkdirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); i++) {
        cur += path[i];
        if (path[i] == '/' || i + 1 == path.size()) mkdir(cur.c_str(), 0755);
    }
}

// src/sim.cu:340-357 on the host (the reference's own order), for rows already on the host.
void robust_host(const std::vector<float>& samples, int pop, int nseeds, std::vector<float>& scores) {
    std::vector<float> row(nseeds);
    int tail_n = (nseeds + 3) / 4;
    for (int i = 0; i < pop; i++) {
        float mean = 0;
        for (int s = 0; s < nseeds; s++) {
            row[s] = samples[(size_t)i * nseeds + s];
            mean += row[s] / nseeds;
        }
        std::sort(row.begin(), row.end());
        float cvar25 = 0;
        for (int s = 0; s < tail_n; s++) cvar25 += row[s] / tail_n;
        scores[i] = 0.65f * mean + 0.25f * cvar25 + 0.10f * row[0];
    }
}

// Device round trip: genomes in, distances (and optionally scores) out.
int eval_host(pe_engine* e, const float* genomes, int pop, const std::vector<int>& seeds,
              std::vector<float>* dist, std::vector<float>* scores) {
    dist->resize((size_t)pop * seeds.size());
    if (scores) scores->resize(pop);
    return pe_evaluate_population(e, genomes, pop, seeds.data(), (int)seeds.size(), 0, PE_MAX_STEPS,
                                  dist->data(), nullptr, scores ? scores->data() : nullptr);
}

// The message pe_last_error() returns, and PE_EINVAL.
int drv_fail(const char* msg) {
    pe::set_last_error(msg);
    return PE_EINVAL;
}

struct EngineGuard {
    pe_engine* e = nullptr;
    ~EngineGuard() { pe_engine_destroy(e); }
};

// A file closed on every return path (close() for the normal one).
struct FileGuard {
    FILE* f = nullptr;
    ~FileGuard() { close(); }
    void close() {
        if (f) fclose(f);
        f = nullptr;
    }
};

inline float gget(const float* g, int i) { return g[i]; }

}  // namespace

extern "C" {

int pe_evaluate_design(const float* genome, int scenarios, int base_seed, const char* csv_path, float* stats) {
    if (!genome) return drv_fail("pe_evaluate_design: NULL genome");
    if (scenarios < 8) scenarios = 8;  // src/sim.cu:259
    EngineGuard eg;
    if (int rc = pe_engine_create(0, &eg.e)) return rc;
    std::vector<int> seeds(scenarios);
    for (int i = 0; i < scenarios; i++) seeds[i] = (int)((uint32_t)base_seed + (uint32_t)i * 7919u);
    // flights and the audit statistics on the device; the distances come back only for the CSV
    std::vector<float> distances(csv_path ? scenarios : 0);
    float st[PE_AUDIT_STATS];
    if (int rc = pe_audit(eg.e, genome, seeds.data(), scenarios, st, csv_path ? distances.data() : nullptr))
        return rc;
    float mp[PE_MASSPROPS_FLOATS], ext[4];
    int nt = 0;
    if (int rc = pe_plane_info(eg.e, 0, mp, ext, &nt)) return rc;  // mass and bounds of the audit line

    if (csv_path) {
        std::string out(csv_path);
        size_t sl = out.find_last_of('/');
        if (sl != std::string::npos && sl > 0) mkdirs(out.substr(0, sl));
        FILE* f = fopen(csv_path, "w");
        if (!f) {
            fprintf(stderr, "cannot write %s\n", csv_path);
        } else {
            fprintf(f, "scenario,seed,distance_m,speed_mps,height_m,pitch_deg,yaw_deg,roll_deg,force_pitch_deg,"
                       "force_yaw_deg,grip_x_mm,grip_y_mm,grip_z_mm,roll_rate,pitch_rate,yaw_rate,air_density,"
                       "skin_cf,gust_scale,base_wind_x,base_wind_y,material_scale,infill_ratio,print_bias_x_mm,"
                       "print_bias_y_mm,print_bias_z_mm,warp_pitch_deg,warp_roll_deg\n");
            const float r2d = 57.2957795131f;
            for (int i = 0; i < scenarios; i++) {
                int seed = seeds[i];
                Scen d = scenario(seed);
                fprintf(f, "%d,%d,%.6f,%.5f,%.5f,%.4f,%.4f,%.4f,%.4f,%.4f,%.3f,%.3f,%.3f,%.5f,%.5f,%.5f,%.6f,%.6f,"
                           "%.6f,%.6f,%.6f,%.5f,%.5f,%.3f,%.3f,%.3f,%.4f,%.4f\n",
                        i, seed, distances[i], d.speed, d.height, d.pitch * r2d, d.yaw * r2d, d.roll * r2d,
                        d.force_pitch * r2d, d.force_yaw * r2d, d.grip_x * 1000, d.grip_y * 1000, d.grip_z * 1000,
                        d.roll_rate, d.pitch_rate, d.yaw_rate, d.air_rho, d.skin_cf, d.gust, d.base_x, d.base_y,
                        d.material_scale, d.infill_ratio, d.bias_x * 1000, d.bias_y * 1000, d.bias_z * 1000,
                        d.warp_pitch * r2d, d.warp_roll * r2d);
            }
            fclose(f);
        }
    }
    // audit, src/sim.cu:291-309 (statistics from pe_distance_stats, the reference's arithmetic)
    printf("robustness audit: %d GPU scenarios -> %s\n", scenarios, csv_path ? csv_path : "(no csv)");
    printf("  min %.2fm  p05 %.2fm  p10 %.2fm  p25 %.2fm  median %.2fm\n", st[0], st[1], st[2], st[3], st[4]);
    printf("  mean %.2fm  sd %.2fm  p75 %.2fm  p90 %.2fm  p95 %.2fm  max %.2fm\n", st[5], st[6], st[7], st[8], st[9],
           st[10]);
    printf("  CVaR10 %.2fm  failures %d/%d  PLA %.1fg  bounds %.0fx%.0fx%.0fmm\n", st[11], (int)st[12], scenarios,
           mp[0] * 1000, ext[0] * 1000, ext[1] * 1000, ext[2] * 1000);
    fflush(stdout);
    if (stats) {
        float s[18];
        memcpy(s, st, sizeof st);
        s[13] = mp[0]; s[14] = ext[0]; s[15] = ext[1]; s[16] = ext[2]; s[17] = (float)scenarios;
        memcpy(stats, s, sizeof s);
    }
    return PE_OK;
}

int pe_select_finalist(const float* candidates, int count, int scenarios, int base_seed, const char* out_dir,
                       int* best_index) {
    if (!candidates || !out_dir) return drv_fail("pe_select_finalist: NULL candidates or output directory");
    if (count < 1 || scenarios < 128) {  // src/sim.cu:360
        fprintf(stderr, "select-best needs candidates>=1 and scenarios>=128\n");
        return drv_fail("select-best needs candidates >= 1 and scenarios >= 128");
    }
    mkdirs(out_dir);
    EngineGuard eg;
    if (int rc = pe_engine_create(0, &eg.e)) return rc;
    std::vector<int> seeds(scenarios);
    for (int i = 0; i < scenarios; i++) seeds[i] = (int)((uint32_t)base_seed + (uint32_t)i * 7919u);
    // every candidate under the same scenario set, one batch (the reference loops candidates)
    std::vector<float> fit;
    if (int rc = eval_host(eg.e, candidates, count, seeds, &fit, nullptr)) return rc;
    std::string csv_path = std::string(out_dir) + "/finalist-selection.csv";
    FileGuard cg;
    cg.f = fopen(csv_path.c_str(), "w");
    if (!cg.f) return drv_fail("cannot create finalist-selection.csv in the output directory");
    FILE* csv = cg.f;
    fprintf(csv, "candidate,robust_score,mean,cvar25,worst\n");
    float best_score = -1e9f;
    int best_i = 0;
    std::vector<float> row(scenarios), score(1), sorted;
    for (int c = 0; c < count; c++) {
        std::copy(fit.begin() + (size_t)c * scenarios, fit.begin() + (size_t)(c + 1) * scenarios, row.begin());
        robust_host(row, 1, scenarios, score);
        sorted = row;
        std::sort(sorted.begin(), sorted.end());
        float mean = 0, cvar = 0;
        int tail = (scenarios + 3) / 4;
        for (float x : sorted) mean += x / scenarios;
        for (int i = 0; i < tail; i++) cvar += sorted[i] / tail;
        fprintf(csv, "%d,%.6f,%.6f,%.6f,%.6f\n", c, score[0], mean, cvar, sorted[0]);
        if (score[0] > best_score) { best_score = score[0]; best_i = c; }
        if (c % 25 == 0 || c == count - 1) {
            printf("finalist %d/%d best %.3fm (candidate %d)\n", c + 1, count, best_score, best_i);
            fflush(stdout);
        }
    }
    cg.close();
    std::string best_path = std::string(out_dir) + "/best-final.bin";
    if (int rc = pe_save_best(best_path.c_str(), candidates + (size_t)best_i * PE_GENOME_FLOATS)) return rc;
    printf("independent finalist winner: candidate %d score %.3fm -> %s\n", best_i, best_score, best_path.c_str());
    if (best_index) *best_index = best_i;
    return PE_OK;
}

int pe_run_ga(int pop, int gens, int nseeds, const char* out_dir, const char* init_path) {
    if (pop < 2 || gens < 1 || nseeds < 1 || !out_dir) {
        fprintf(stderr, "evolve requires pop>=2, gens>=1, seeds>=1\n");
        return drv_fail("evolve requires pop >= 2, gens >= 1, seeds >= 1 and an output directory");
    }
    const int G = PE_GENOME_FLOATS;
    mkdirs(out_dir);
    float lo[G], hi[G];
    pe_genome_bounds(lo, hi);
    auto gset = [&](float* g, int i, float v) { g[i] = fminf(hi[i], fmaxf(lo[i], v)); };
    std::mt19937 rng(42);
    std::uniform_real_distribution<float> u01(0, 1);
    auto grand = [&](float* g) {
        std::uniform_real_distribution<float> u(0, 1);
        for (int i = 0; i < G; i++) gset(g, i, lo[i] + u(rng) * (hi[i] - lo[i]));
    };
    std::vector<float> gs((size_t)pop * G), next((size_t)pop * G);
    for (int k = 0; k < pop; k++) grand(&gs[(size_t)k * G]);
    if (init_path) {
        int n = 0;
        std::vector<float> warm((size_t)pop * G);
        if (pe_load_genomes(init_path, warm.data(), pop, &n) == PE_OK) {
            n = std::min(n, pop);
            std::copy(warm.begin(), warm.begin() + (size_t)n * G, gs.begin());
            pe_sanitize_genomes(gs.data(), n);
            printf("warm start: %d genomes from %s (clamped to printable bounds)\n", n, init_path);
        }
    }
    EngineGuard eg, ev;
    if (int rc = pe_engine_create(0, &eg.e)) return rc;
    if (int rc = pe_engine_create(0, &ev.e)) return rc;
    const int VAL_N = 128;
    std::vector<int> val_seeds(VAL_N);  // holdout: gpu_sim(128 copies, 100003, vary 1)
    for (int i = 0; i < VAL_N; i++) val_seeds[i] = 100003 + i * 7919;
    std::vector<float> samples, acc, val_fit, val_score(1);
    std::vector<int> idx(pop);
    std::vector<float> best_ever(G, 0.0f);
    float best_ever_f = -1e9f;
    std::vector<float> archive;
    std::string od(out_dir);
    FileGuard hg;
    hg.f = fopen((od + "/history.csv").c_str(), "w");
    if (!hg.f) return drv_fail("cannot create history.csv in the output directory");
    FILE* hist = hg.f;
    fprintf(hist, "gen,train_best,holdout128,mean,p90\n");
    std::normal_distribution<float> nrm(0, 1);
    std::vector<int> seeds(nseeds);
    auto sort_idx = [&]() {
        for (int i = 0; i < pop; i++) idx[i] = i;
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return acc[a] > acc[b]; });
    };
    for (int gen = 0; gen < gens; gen++) {
        for (int s = 0; s < nseeds; s++) seeds[s] = gen * nseeds + s + 1;
        if (int rc = eval_host(eg.e, gs.data(), pop, seeds, &samples, &acc)) return rc;
        sort_idx();
        float mean = 0;
        for (int i = 0; i < pop; i++) mean += acc[i] / pop;
        int val_k = std::min(8, pop);
        float holdout = -1e9f;
        int champion_i = idx[0];
        std::vector<float> cands((size_t)val_k * G);
        for (int c = 0; c < val_k; c++) std::copy(&gs[(size_t)idx[c] * G], &gs[(size_t)idx[c] * G] + G, &cands[(size_t)c * G]);
        std::vector<float> vdist;
        if (int rc = eval_host(ev.e, cands.data(), val_k, val_seeds, &vdist, nullptr)) return rc;
        for (int c = 0; c < val_k; c++) {
            val_fit.assign(vdist.begin() + (size_t)c * VAL_N, vdist.begin() + (size_t)(c + 1) * VAL_N);
            robust_host(val_fit, 1, VAL_N, val_score);
            if (val_score[0] > holdout) { holdout = val_score[0]; champion_i = idx[c]; }
        }
        fprintf(hist, "%d,%.3f,%.3f,%.3f,%.3f\n", gen, acc[idx[0]], holdout, mean, acc[idx[pop / 10]]);
        fflush(hist);
        if (gen % 10 == 0 || gen == gens - 1)
            printf("gen %4d train %7.2fm holdout %7.2fm mean %7.2fm p90 %7.2fm\n", gen, acc[idx[0]], holdout, mean,
                   acc[idx[pop / 10]]);
        if (holdout > best_ever_f) {
            best_ever_f = holdout;
            std::copy(&gs[(size_t)champion_i * G], &gs[(size_t)champion_i * G] + G, best_ever.begin());
        }
        archive.insert(archive.end(), &gs[(size_t)champion_i * G], &gs[(size_t)champion_i * G] + G);
        if (gen % 25 == 24) {  // checkpoint, src/sim.cu:464-470
            pe_save_best((od + "/best.bin").c_str(), best_ever.data());
            std::vector<float> srt((size_t)pop * G);
            for (int i = 0; i < pop; i++) std::copy(&gs[(size_t)idx[i] * G], &gs[(size_t)idx[i] * G] + G, &srt[(size_t)i * G]);
            pe_save_genomes((od + "/pop.bin").c_str(), srt.data(), pop);
            pe_save_genomes((od + "/archive.bin").c_str(), archive.data(), (int)(archive.size() / G));
        }
        // evolve, src/sim.cu:472-490
        int elite = pop / 64;
        float anneal = 1.0f - 0.6f * gen / gens;
        for (int i = 0; i < elite; i++) std::copy(&gs[(size_t)idx[i] * G], &gs[(size_t)idx[i] * G] + G, &next[(size_t)i * G]);
        for (int i = elite; i < pop; i++) {
            float* ni = &next[(size_t)i * G];
            if (u01(rng) < 0.05f) { grand(ni); continue; }
            auto tourn = [&]() {
                int b = idx[(int)(u01(rng) * pop)];
                for (int k = 0; k < 3; k++) {
                    int c = (int)(u01(rng) * pop);
                    if (acc[c] > acc[b]) b = c;
                }
                return b;
            };
            int ia = tourn();
            int ic = tourn();
            const float* pa = &gs[(size_t)ia * G];
            const float* pc = &gs[(size_t)ic * G];
            float tmp[G];
            for (int j = 0; j < G; j++) {
                float a = -0.1f + 1.2f * u01(rng);
                float v = gget(pa, j) * a + gget(pc, j) * (1 - a);
                if (u01(rng) < 0.25f) v += nrm(rng) * 0.08f * (hi[j] - lo[j]) * anneal;
                gset(tmp, j, v);
            }
            std::copy(tmp, tmp + G, ni);
        }
        gs.swap(next);
    }
    hg.close();
    if (int rc = pe_save_best((od + "/best.bin").c_str(), best_ever.data())) return rc;
    for (int s = 0; s < nseeds; s++) seeds[s] = 777 + s;  // final re-evaluation, src/sim.cu:495-502
    if (int rc = eval_host(eg.e, gs.data(), pop, seeds, &samples, &acc)) return rc;
    sort_idx();
    std::vector<float> srt((size_t)pop * G);
    for (int i = 0; i < pop; i++) std::copy(&gs[(size_t)idx[i] * G], &gs[(size_t)idx[i] * G] + G, &srt[(size_t)i * G]);
    if (int rc = pe_save_genomes((od + "/pop.bin").c_str(), srt.data(), pop)) return rc;
    if (int rc = pe_save_genomes((od + "/archive.bin").c_str(), archive.data(), (int)(archive.size() / G))) return rc;
    printf("best holdout score: %.2fm (saved %s/best.bin)\n", best_ever_f, out_dir);
    const float* bg = best_ever.data();
    printf("genome: span=%.3f chord=%.3f taper=%.2f sweep=%.2f dih_in=%.2f dih_out=%.2f kink=%.2f\n"
           "        camber=(%.3f,%.3f) washout=%.3f elev=%.3f nose=%.2f keel=%.3f deck=(%.3f,%.2f) body=%.2f\n"
           "        fin=(h %.3f, chord %.2f, sweep %.2f) tail=(span %.2f, chord %.2f, angle %.3f)\n",
           bg[0], bg[1], bg[2], bg[3], bg[4], bg[5], bg[6], bg[7], bg[8], bg[9], bg[10], bg[11], bg[12], bg[13],
           bg[14], bg[15], bg[16], bg[17], bg[18], bg[19], bg[20], bg[21]);
    fflush(stdout);
    return PE_OK;
}

}  // extern "C"
