// grad_host_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Instantiates the product's differentiable model (planes-rl_gb300/csrc/pe_grad_model.h) in
// double on the host, so the CPU tests can check its adjoint against FP64 central finite
// differences of the oracle's smoothed landing distance.  Built by tests/conftest.py into
// tests/_build/libgrad_host.so.
#include <cstdint>
#include <memory>
#include <vector>

#include "../planes-rl_gb300/csrc/pe_grad_model.h"

using namespace pg;

namespace {
double seed_phase_d(int seed) {  // src/common.h:371-374
    int32_t prod = (int32_t)((uint32_t)seed * 37u);
    return (double)(prod % 97);
}

// Mesh, mass properties and panels of a genome in T; returns printability.
template <class T>
int make_plane(const float* genome, PlaneData<T>& pd, V3<T>* com_out) {
    T g[35];
    for (int k = 0; k < 35; k++) g[k] = genome[k];
    std::vector<V3<T>> V(kNvMax);
    V3<T> com;
    plane_data(g, V.data(), &pd.mass, pd.I, &com, &pd.nt);
    Topo tp = topology(g);
    V3<T> lo = V[0], hi = V[0];
    for (int i = 1; i < tp.nv; i++) {
        lo = v3(p_min(lo.x, V[i].x), p_min(lo.y, V[i].y), p_min(lo.z, V[i].z));
        hi = v3(p_max(hi.x, V[i].x), p_max(hi.y, V[i].y), p_max(hi.z, V[i].z));
    }
    const T lim = (T)(0.250f - 0.00045f);
    int printable = (hi.x - lo.x) <= lim && (hi.y - lo.y) <= lim && (hi.z - lo.z) <= lim;
    for (int t = 0; t < pd.nt; t++) panel(V.data(), tp, com, t, &pd.c[t], &pd.A[t], &pd.n[t]);
    if (com_out) *com_out = com;
    return printable;
}
}  // namespace

extern "C" {

// Plane data of one genome: mass, I[6], com[3], panels c[nt][3], A[nt], n[nt][3].
int pgh_plane_data(const float* genome, double* mass, double* I6, double* com, double* c, double* A, double* n,
                   int* nt) {
    auto pd = std::make_unique<PlaneData<double>>();
    V3<double> cm;
    int printable = make_plane(genome, *pd, &cm);
    *mass = pd->mass;
    for (int q = 0; q < 6; q++) I6[q] = pd->I[q];
    com[0] = cm.x; com[1] = cm.y; com[2] = cm.z;
    *nt = pd->nt;
    for (int t = 0; t < pd->nt; t++) {
        c[t * 3] = pd->c[t].x; c[t * 3 + 1] = pd->c[t].y; c[t * 3 + 2] = pd->c[t].z;
        A[t] = pd->A[t];
        n[t * 3] = pd->n[t].x; n[t * 3 + 1] = pd->n[t].y; n[t * 3 + 2] = pd->n[t].z;
    }
    return printable;
}

// One flight on given plane data: its smoothed distance and the adjoint wrt that plane data.
double pgh_flight(const double* scen, int seed, double mass, const double* I6, int nt, const double* c,
                  const double* A, const double* n, int max_steps, int K, int* kind, int* steps, double* Lmass,
                  double* LI6, double* Lc, double* LA, double* Ln) {
    auto pd = std::make_unique<PlaneData<double>>();
    auto out = std::make_unique<PlaneAdj<double>>();
    pd->mass = mass;
    for (int q = 0; q < 6; q++) pd->I[q] = I6[q];
    pd->nt = nt;
    for (int t = 0; t < nt; t++) {
        pd->c[t] = v3(c[t * 3], c[t * 3 + 1], c[t * 3 + 2]);
        pd->A[t] = A[t];
        pd->n[t] = v3(n[t * 3], n[t * 3 + 1], n[t * 3 + 2]);
    }
    std::vector<St<double>> ck(max_steps / K + 2);
    double d = flight_grad_serial(scen, seed_phase_d(seed), *pd, max_steps, K, *out, kind, steps, ck.data());
    *Lmass = out->mass;
    for (int q = 0; q < 6; q++) LI6[q] = out->I[q];
    for (int t = 0; t < nt; t++) {
        Lc[t * 3] = out->c[t].x; Lc[t * 3 + 1] = out->c[t].y; Lc[t * 3 + 2] = out->c[t].z;
        LA[t] = out->A[t];
        Ln[t * 3] = out->n[t].x; Ln[t * 3 + 1] = out->n[t].y; Ln[t * 3 + 2] = out->n[t].z;
    }
    return d;
}

}  // extern "C"

// The tail-aware objective of one genome over S scenarios (scen [S][25] in double, as the
// oracle's scenario draw gives them) and its gradient wrt the 35 genes, computed in T.
template <class T>
int objective_grad(const float* genome, const double* scen_d, const int* seeds, int S, int max_steps, int K,
                   double* J, double* grad, double* d_out, int* kind_out, int* steps_out) {
    auto pd = std::make_unique<PlaneData<T>>();
    int printable = make_plane(genome, *pd, (V3<T>*)nullptr);
    for (int j = 0; j < 35; j++) grad[j] = 0;
    if (!printable) {
        for (int s = 0; s < S; s++) { d_out[s] = -100; kind_out[s] = 0; steps_out[s] = 0; }
        *J = -100;
        return 0;
    }
    std::vector<T> scen(25 * S), d(S);
    for (int k = 0; k < 25 * S; k++) scen[k] = (T)scen_d[k];
    std::vector<std::unique_ptr<PlaneAdj<T>>> adj;
    std::vector<St<T>> ck(max_steps / K + 2);
    for (int s = 0; s < S; s++) {
        adj.emplace_back(new PlaneAdj<T>());
        d[s] = flight_grad_serial(scen.data() + 25 * s, (T)seed_phase_d(seeds[s]), *pd, max_steps, K, *adj.back(),
                                  &kind_out[s], &steps_out[s], ck.data());
        d_out[s] = d[s];
    }
    std::vector<T> w(S);
    *J = objective_weights(d.data(), S, w.data());
    auto ybar = std::make_unique<PlaneAdj<T>>();
    ybar->mass = 0;
    for (int q = 0; q < 6; q++) ybar->I[q] = 0;
    for (int t = 0; t < pd->nt; t++) { ybar->c[t] = v3(T(0), T(0), T(0)); ybar->n[t] = ybar->c[t]; ybar->A[t] = 0; }
    for (int s = 0; s < S; s++) {
        const PlaneAdj<T>& a = *adj[s];
        ybar->mass += w[s] * a.mass;
        for (int q = 0; q < 6; q++) ybar->I[q] += w[s] * a.I[q];
        for (int t = 0; t < pd->nt; t++) {
            ybar->c[t] = ybar->c[t] + a.c[t] * w[s];
            ybar->n[t] = ybar->n[t] + a.n[t] * w[s];
            ybar->A[t] += w[s] * a.A[t];
        }
    }
    std::vector<V3<Dual<T>>> Vbuf(kNvMax);
    for (int j = 0; j < 35; j++) grad[j] = (double)genome_jvp(genome, j, *ybar, Vbuf.data());
    return 1;
}

extern "C" {
int pgh_objective_grad(const float* genome, const double* scen, const int* seeds, int S, int max_steps, int K,
                       double* J, double* grad, double* d_out, int* kind_out, int* steps_out) {
    return objective_grad<double>(genome, scen, seeds, S, max_steps, K, J, grad, d_out, kind_out, steps_out);
}
// The same in float arithmetic (the precision of the GPU kernels).
int pgh_objective_grad_f32(const float* genome, const double* scen, const int* seeds, int S, int max_steps, int K,
                           double* J, double* grad, double* d_out, int* kind_out, int* steps_out) {
    return objective_grad<float>(genome, scen, seeds, S, max_steps, K, J, grad, d_out, kind_out, steps_out);
}
}  // extern "C"
