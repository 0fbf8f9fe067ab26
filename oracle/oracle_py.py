"""ctypes wrapper of oracle/_build/liboracle.so -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the oracle; the
product never imports it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_build():
    import importlib.util

    spec = importlib.util.spec_from_file_location("planes_oracle_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_build = _load_build()

MAX_V, MAX_T, MP_N, SCEN_N, STATE_N = 512, 900, 20, 25, 16

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build_oracle())
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dt(prec):
    return np.float32 if prec == 32 else np.float64


def _fn(prec, name):
    return getattr(lib(), ("orf_" if prec == 32 else "ord_") + name)


def genome_bounds():
    lo = np.zeros(35, np.float32)
    hi = np.zeros(35, np.float32)
    lib().or_genome_bounds(_p(lo), _p(hi))
    return lo, hi


def grand(seed, n):
    """Genomes drawn like the reference's grand() from std::mt19937(seed)."""
    g = np.zeros((n, 35), np.float32)
    lib().or_grand(C.c_uint32(seed), n, _p(g))
    return g


def build_mesh(genome, prec=32):
    V = np.zeros((MAX_V, 3), _dt(prec))
    T = np.zeros((MAX_T, 3), np.int32)
    nv, nt = C.c_int(), C.c_int()
    g = np.ascontiguousarray(genome, np.float32)
    _fn(prec, "build_mesh")(_p(g), _p(V), _p(T), C.byref(nv), C.byref(nt))
    return V[:nv.value].copy(), T[:nt.value].copy()


def fits_print_volume(V, prec=32):
    V = np.ascontiguousarray(V, _dt(prec))
    return bool(_fn(prec, "fits_print_volume")(_p(V), V.shape[0]))


def mesh_extent(V, prec=32):
    V = np.ascontiguousarray(V, _dt(prec))
    e = np.zeros(3, _dt(prec))
    _fn(prec, "mesh_extent")(_p(V), V.shape[0], _p(e))
    return e


def mass_props(genome, V, T, prec=32):
    g = np.ascontiguousarray(genome, np.float32)
    V = np.ascontiguousarray(V, _dt(prec))
    T = np.ascontiguousarray(T, np.int32)
    mp = np.zeros(MP_N, _dt(prec))
    _fn(prec, "mass_props")(_p(g), _p(V), _p(T), T.shape[0], _p(mp))
    return mp


def scenario_desc(seed, prec=32):
    d = np.zeros(SCEN_N, _dt(prec))
    _fn(prec, "scenario_desc")(int(seed), _p(d))
    return d


def printed_mass_props(mp, d, prec=32):
    mp = np.ascontiguousarray(mp, _dt(prec))
    d = np.ascontiguousarray(d, _dt(prec))
    out = np.zeros(MP_N, _dt(prec))
    cg = np.zeros(3, _dt(prec))
    _fn(prec, "printed_mass_props")(_p(mp), _p(d), _p(out), _p(cg))
    return out, cg


def wind_at(p, t, seed, prec=32):
    p = np.ascontiguousarray(p, _dt(prec))
    out = np.zeros(3, _dt(prec))
    ft = C.c_float if prec == 32 else C.c_double
    f = _fn(prec, "wind_at")
    f.argtypes = [C.c_void_p, ft, C.c_int, C.c_void_p]
    f(_p(p), t, int(seed), _p(out))
    return out


class Prepared:
    """Panels and mass properties of a population, as k_prepare leaves them (MAX_T stride)."""

    def __init__(self, genomes, prec=32):
        g = np.ascontiguousarray(genomes, np.float32)
        self.pop = g.shape[0]
        self.prec = prec
        dt = _dt(prec)
        self.pc = np.zeros((self.pop, MAX_T, 4), dt)
        self.pn = np.zeros((self.pop, MAX_T, 4), dt)
        self.mp = np.zeros((self.pop, MP_N), dt)
        self.nt = np.zeros(self.pop, np.int32)
        _fn(prec, "prepare")(_p(g), self.pop, _p(self.pc), _p(self.pn), _p(self.mp), _p(self.nt))

    def release(self, p, env_seed):
        st = np.zeros(STATE_N, _dt(self.prec))
        _fn(self.prec, "release")(_p(self.mp[p]), int(self.nt[p]), int(env_seed), _p(st))
        return st

    def step(self, p, env_seed, state, step, max_steps=7200):
        dt = _dt(self.prec)
        st = np.ascontiguousarray(state, dt)
        out = np.zeros(STATE_N, dt)
        ft = np.zeros(6, dt)
        _fn(self.prec, "step")(_p(self.pc[p]), _p(self.pn[p]), int(self.nt[p]), _p(self.mp[p]), int(env_seed),
                               _p(st), int(step), int(max_steps), _p(out), _p(ft))
        return out, ft

    def fly(self, p, env_seed, max_steps=7200):
        fit = (C.c_float if self.prec == 32 else C.c_double)()
        n = C.c_int()
        st = np.zeros(STATE_N, _dt(self.prec))
        _fn(self.prec, "fly")(_p(self.pc[p]), _p(self.pn[p]), int(self.nt[p]), _p(self.mp[p]), int(env_seed),
                              int(max_steps), C.byref(fit), C.byref(n), _p(st))
        return fit.value, n.value, st

    def fly_rec(self, p, env_seed, spread, rec_every, rec_cap, grid_index=None):
        """The reference's gpu_sim for plane p with recording: (rec [rec_cap][8], fitness)."""
        dt = _dt(self.prec)
        rec = np.full((rec_cap, 8), np.nan, dt)  # slots the loop never reaches stay NaN
        fit = (C.c_float if self.prec == 32 else C.c_double)()
        _fn(self.prec, "fly_rec")(_p(self.pc[p]), _p(self.pn[p]), int(self.nt[p]), _p(self.mp[p]), int(env_seed),
                                  int(p if grid_index is None else grid_index),
                                  (C.c_float if self.prec == 32 else C.c_double)(spread), int(rec_every),
                                  int(rec_cap), _p(rec), C.byref(fit))
        return rec, fit.value

    def fly_smooth(self, p, env_seed, max_steps=7200):
        d = (C.c_float if self.prec == 32 else C.c_double)()
        n, kind = C.c_int(), C.c_int()
        _fn(self.prec, "fly_smooth")(_p(self.pc[p]), _p(self.pn[p]), int(self.nt[p]), _p(self.mp[p]), int(env_seed),
                                     int(max_steps), C.byref(d), C.byref(n), C.byref(kind))
        return d.value, n.value, kind.value

    def eval(self, seeds, vary=0, max_steps=7200, nthreads=None):
        seeds = np.ascontiguousarray(seeds, np.int32)
        S = seeds.size
        dist = np.zeros(self.pop * S, _dt(self.prec))
        steps = np.zeros(self.pop * S, np.int32)
        nthreads = nthreads or os.cpu_count() or 1
        _fn(self.prec, "eval_prepared")(_p(self.pc), _p(self.pn), _p(self.mp), _p(self.nt), self.pop, _p(seeds), S,
                                        int(vary), int(max_steps), _p(dist), _p(steps), int(nthreads))
        return dist, steps


def eval_batch(genomes, seeds, vary=0, max_steps=7200, prec=32, nthreads=None):
    """Whole fitness path on the host: prepare + every flight.  Returns (dist, steps)."""
    g = np.ascontiguousarray(genomes, np.float32)
    seeds = np.ascontiguousarray(seeds, np.int32)
    pop, S = g.shape[0], seeds.size
    dist = np.zeros(pop * S, _dt(prec))
    steps = np.zeros(pop * S, np.int32)
    nthreads = nthreads or os.cpu_count() or 1
    _fn(prec, "eval_batch")(_p(g), pop, _p(seeds), S, int(vary), int(max_steps), _p(dist), _p(steps), int(nthreads))
    return dist, steps


def robust_scores(samples, pop, nseeds):
    s = np.ascontiguousarray(samples, np.float32).reshape(-1)
    out = np.zeros(pop, np.float32)
    lib().or_robust_scores(_p(s), pop, nseeds, _p(out))
    return out


def audit_stats(dist):
    """The robustness audit's 13 statistics of a distance vector (or_audit_stats)."""
    d = np.ascontiguousarray(dist, np.float32).reshape(-1)
    out = np.zeros(13, np.float32)
    lib().or_audit_stats(_p(d), d.size, _p(out))
    return out


def env_seed(seed, p, vary):
    return int(np.int32(np.uint32(seed) + (np.uint32(p) * np.uint32(7919) if vary else np.uint32(0))))


def tail_objective(d):
    """0.65 mean + 0.25 mean(worst ceil(S/4)) + 0.10 min over one genome's distances (double)."""
    d = np.asarray(d, np.float64)
    S = d.size
    tail = (S + 3) // 4
    srt = np.sort(d)
    return 0.65 * d.mean() + 0.25 * srt[:tail].mean() + 0.10 * srt[0]


def smooth_objective(genome, seeds, max_steps=7200):
    """FP64 oracle: the tail-aware objective of one genome over smoothed landing distances."""
    pre = Prepared(np.asarray(genome, np.float32)[None], prec=64)
    d = [pre.fly_smooth(0, int(s), max_steps)[0] for s in seeds]
    return tail_objective(d), np.array(d)
