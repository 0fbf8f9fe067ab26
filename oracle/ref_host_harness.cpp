// ref_host_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C-ABI shim over the reference's own src/common.h, compiled by oracle/build.py straight from
// the reference tree (its path is given with -I; no reference source is copied here).  It lets
// tests/golden/make_host_golden.py record the reference's mesher, mass properties, scenario
// draw, print variation and gust field as golden vectors that pin the C oracle bit-for-bit.
#include "common.h"

#include <string.h>

extern void write_presets(const char* out_dir, float thickness_mm);  // src/designs.cu:58

extern "C" {

int ref_sizes(int* out) {
    out[0] = (int)sizeof(Genome);
    out[1] = (int)sizeof(MassProps);
    out[2] = (int)sizeof(ScenarioDesc);
    out[3] = (int)sizeof(PlaneState);
    out[4] = MAX_V;
    out[5] = MAX_T;
    return 0;
}

int ref_build_mesh(const float* genome, float* V, int* T, int* nv, int* nt) {
    static v3 VV[MAX_V];
    static int TT[MAX_T][3];
    Genome g;
    memcpy(&g, genome, sizeof g);
    MeshOut mo;
    build_mesh(&g, VV, TT, &mo);
    memcpy(V, VV, sizeof(v3) * mo.nv);
    memcpy(T, TT, sizeof(int) * 3 * mo.nt);
    *nv = mo.nv;
    *nt = mo.nt;
    return 0;
}

int ref_fits_print_volume(const float* V, int nv) {
    return fits_print_volume((const v3*)V, nv, PRINT_VOLUME_M - PLA_WALL_M);
}

void ref_mesh_extent(const float* V, int nv, float* ext) {
    v3 e = mesh_extent((const v3*)V, nv);
    ext[0] = e.x; ext[1] = e.y; ext[2] = e.z;
}

void ref_mass_props(const float* genome, const float* V, const int* T, int nt, float* mp) {
    Genome g;
    memcpy(&g, genome, sizeof g);
    MassProps m;
    mass_props(&g, (const v3*)V, (const int(*)[3])T, nt, &m);
    memcpy(mp, &m, sizeof m);
}

void ref_scenario_desc(int seed, float* d) {
    ScenarioDesc s = scenario_desc(seed);
    memcpy(d, &s, sizeof s);
}

void ref_printed_mass_props(const float* mp, const float* d, float* out, float* cg) {
    MassProps m;
    ScenarioDesc s;
    memcpy(&m, mp, sizeof m);
    memcpy(&s, d, sizeof s);
    v3 shift;
    MassProps r = printed_mass_props(m, s, &shift);
    memcpy(out, &r, sizeof r);
    cg[0] = shift.x; cg[1] = shift.y; cg[2] = shift.z;
}

void ref_wind_at(const float* p, float t, int seed, float* out) {
    v3 w = wind_at(V3(p[0], p[1], p[2]), t, seed);
    out[0] = w.x; out[1] = w.y; out[2] = w.z;
}

int ref_write_presets(const char* dir) {
    write_presets(dir, 0.45f);
    return 0;
}

}  // extern "C"
