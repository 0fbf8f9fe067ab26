// pe_cli.cpp -- `planes`: the reference's command line (src/main.cu:36-106) for the modes that
// run the fitness path: evolve, evaluate, select-best.  Same flags and defaults.  The video,
// STL and preset modes belong to the reference's renderer / exporters and are not part of this
// build.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "planes_eval.h"

static const char* opt(int argc, char** argv, const char* key, const char* dflt) {
    for (int i = 2; i < argc - 1; i++)
        if (!strcmp(argv[i], key)) return argv[i + 1];
    return dflt;
}

static int usage() {
    printf("usage: planes <evolve|evaluate|select-best> [opts]\n"
           "  evolve    --pop 4096 --gens 400 --seeds 8 --out out [--init out/pop.bin]\n"
           "  evaluate  --best out/best.bin --n 512 --seed 9001 --o out/robustness.csv\n"
           "  select-best --pop-file out/archive.bin --n 8192 --seed 1900001 --out out/run\n");
    return 1;
}

static int report(int rc) {
    if (rc != PE_OK) fprintf(stderr, "planes: error %d: %s\n", rc, pe_last_error());
    return rc == PE_OK ? 0 : 1;
}

int main(int argc, char** argv) {
    if (argc < 2) return usage();
    const char* mode = argv[1];
    if (!strcmp(mode, "evolve")) {
        return report(pe_run_ga(atoi(opt(argc, argv, "--pop", "4096")), atoi(opt(argc, argv, "--gens", "400")),
                                atoi(opt(argc, argv, "--seeds", "3")), opt(argc, argv, "--out", "out"),
                                opt(argc, argv, "--init", nullptr)));
    }
    if (!strcmp(mode, "evaluate")) {
        float g[PE_GENOME_FLOATS];
        const char* path = opt(argc, argv, "--best", "out/best.bin");
        if (pe_load_best(path, g) != PE_OK) {
            fprintf(stderr, "missing %s\n", path);
            return 1;
        }
        return report(pe_evaluate_design(g, atoi(opt(argc, argv, "--n", "512")), atoi(opt(argc, argv, "--seed", "9001")),
                                         opt(argc, argv, "--o", "out/robustness.csv"), nullptr));
    }
    if (!strcmp(mode, "select-best")) {
        const char* path = opt(argc, argv, "--pop-file", "out/archive.bin");
        int n = 0;
        if (pe_load_genomes(path, nullptr, 0, &n) != PE_OK) {
            fprintf(stderr, "missing %s\n", path);
            return 1;
        }
        std::vector<float> gs((size_t)n * PE_GENOME_FLOATS);
        if (pe_load_genomes(path, gs.data(), n, &n) != PE_OK) {
            fprintf(stderr, "truncated %s\n", path);
            return 1;
        }
        return report(pe_select_finalist(gs.data(), n, atoi(opt(argc, argv, "--n", "8192")),
                                         atoi(opt(argc, argv, "--seed", "1900001")), opt(argc, argv, "--out", "out"),
                                         nullptr));
    }
    static const char* other[] = {"showcase", "hero", "robust-video", "evolution-video", "turntable", "stl",
                                  "inspect", "presets"};
    for (const char* o : other)
        if (!strcmp(mode, o)) {
            fprintf(stderr, "planes: mode %s belongs to the renderer / exporters, which this build does not include\n", mode);
            return 1;
        }
    fprintf(stderr, "unknown mode %s\n", mode);
    return 1;
}
