"""ctypes binding of include/planes_eval.h (libplanes_gb300.so).

This is how the Python side of the repository (tests, bench, smoke) calls the CUDA path.  It
mirrors the reference's evaluation boundary (src/sim.h:9-13) and adds the batched engine.
There is no fallback: if the shared library is missing or fails to load, import raises.

Device buffers are passed as integer addresses (e.g. torch.Tensor.data_ptr()); host buffers
as numpy arrays.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libplanes_gb300.so")

PE_OK, PE_EINVAL, PE_ENOMEM, PE_ECUDA, PE_ENOTSUP, PE_ENODEV = 0, 1, 2, 3, 4, 5
MAX_POP = 4194304  # PE_MAX_POP: planes per call (32-bit panel offsets)
GENOME_FLOATS = 35
MP_FLOATS = 20
STATE_FLOATS = 16
MAX_STEPS = 7200


class PEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("planes_eval error %d: %s" % (code, msg))
        self.code = code


class EvolveConfig(C.Structure):
    _fields_ = [("pop", C.c_int), ("gens", C.c_int), ("nseeds", C.c_int), ("seed", C.c_uint), ("max_steps", C.c_int),
                ("polish_top", C.c_int), ("polish_steps", C.c_int), ("polish_lr", C.c_float),
                ("polish_max_steps", C.c_int), ("holdout", C.c_int), ("holdout_base", C.c_int), ("audit", C.c_int),
                ("audit_base", C.c_int)]


class EvolveResult(C.Structure):
    _fields_ = [("best_genome", C.c_float * 35), ("best_holdout", C.c_float), ("best_gen", C.c_int),
                ("audit_score", C.c_float), ("gpu_seconds", C.c_double), ("grad_calls", C.c_int)]


class Config(C.Structure):
    _fields_ = [("lanes", C.c_int), ("warps", C.c_int), ("chunk", C.c_int), ("blocks", C.c_int),
                ("use_graph", C.c_int), ("formulation", C.c_int), ("reg_cap", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_VP = C.c_void_p
_I = C.c_int
# name -> (restype, argtypes)
SIGNATURES = {
    "pe_last_error": (C.c_char_p, []),
    "pe_version": (_I, []),
    "pe_panelbuf_alloc": (_I, [_I, C.POINTER(_VP)]),
    "pe_panelbuf_free": (_I, [_VP]),
    "pe_prepare": (_I, [_VP, _VP, _I, _VP]),
    "pe_sim": (_I, [_VP, _I, _I, _VP, _VP, _I, _I, C.c_float, _I, _VP]),
    "pe_engine_create": (_I, [_I, C.POINTER(_VP)]),
    "pe_engine_destroy": (_I, [_VP]),
    "pe_engine_get_config": (_I, [_VP, C.POINTER(Config)]),
    "pe_engine_set_config": (_I, [_VP, C.POINTER(Config)]),
    "pe_eval_batch": (_I, [_VP, _VP, _I, _VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    "pe_engine_set_smooth_landing": (_I, [_VP, _I]),
    "pe_evaluate_population": (_I, [_VP, _VP, _I, _VP, _I, _I, _I, _VP, _VP, _VP]),
    "pe_robust_scores": (_I, [_VP, _I, _I, _VP, _VP]),
    "pe_distance_stats": (_I, [_VP, _I, _VP, _VP]),
    "pe_audit": (_I, [_VP, _VP, _VP, _I, _VP, _VP]),
    "pe_grad": (_I, [_VP, _VP, _I, _VP, _I, _I, _I, _I, _VP, _VP, _VP, _VP]),
    "pe_objective": (_I, [_VP, _VP, _I, _VP, _I, _I, _I, _I, _VP, _VP, _VP]),
    "pe_topk": (_I, [_VP, _I, _I, _VP, _VP, _VP]),
    "pe_select_top": (_I, [_VP, _VP, _I, _I, _VP, _VP, _VP]),
    "pe_ga_step": (_I, [_VP, _VP, _I, _I, _I, C.c_ulonglong, _VP, _VP]),
    "pe_evolve": (_I, [_VP, C.POINTER(EvolveConfig), _VP, C.POINTER(EvolveResult)]),
    "pe_plane_table": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(_I), _VP]),
    "pe_autotune": (_I, [_VP, _VP, _I, _VP, _I, _I, _I, C.POINTER(Config)]),
    "pe_last_timing": (_I, [_VP, _VP, C.POINTER(_I)]),
    "pe_debug_release": (_I, [_VP, _I, _VP, _I, _I, _VP, _VP]),
    "pe_debug_step": (_I, [_VP, _I, _VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _I, _I, _VP]),
    "pe_debug_station_mode": (_I, [_I]),
    "pe_debug_fail_evaluations": (_I, [_I]),
    "pe_genome_bounds": (_I, [_VP, _VP]),
    "pe_random_genomes": (_I, [C.c_uint, _I, _VP]),
    "pe_sanitize_genomes": (_I, [_VP, _I]),
    "pe_save_best": (_I, [C.c_char_p, _VP]),
    "pe_load_best": (_I, [C.c_char_p, _VP]),
    "pe_save_genomes": (_I, [C.c_char_p, _VP, _I]),
    "pe_load_genomes": (_I, [C.c_char_p, _VP, _I, C.POINTER(_I)]),
    "pe_fp32_peak_probe": (_I, [_I, C.POINTER(C.c_float)]),
    "pe_eval_batch_noalloc": (_I, [_VP, _I, _VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
}


def load(path=LIB_PATH):
    if not os.path.exists(path):
        raise OSError("libplanes_gb300.so not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


LIB = load()


def _check(rc):
    if rc != PE_OK:
        raise PEError(rc, LIB.pe_last_error().decode())


def _ptr(a):
    """Address of a numpy array, a torch tensor or an int (device address); None -> NULL."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    return a.data_ptr()  # torch tensor (device or pinned host)


def _seeds(seeds):
    s = np.ascontiguousarray(np.asarray(seeds, dtype=np.int32).reshape(-1))
    return s, s.ctypes.data, int(s.size)


class Engine:
    """Batched evaluator on one GPU (pe_engine)."""

    def __init__(self, device=0):
        h = _VP()
        _check(LIB.pe_engine_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            LIB.pe_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def config(self):
        c = Config()
        _check(LIB.pe_engine_get_config(self.h, C.byref(c)))
        return c

    def set_config(self, **kw):
        c = self.config
        for k, v in kw.items():
            setattr(c, k, int(v))
        _check(LIB.pe_engine_set_config(self.h, C.byref(c)))
        return c

    def set_smooth_landing(self, on):
        """Report the z = 0 crossing interpolated between the last two states (pe_grad's distance)
        instead of the reference's last x, for this engine's later evaluations."""
        _check(LIB.pe_engine_set_smooth_landing(self.h, 1 if on else 0))

    def eval_batch(self, d_genomes, pop, seeds, vary=0, max_steps=MAX_STEPS, d_dist=None, d_steps=None,
                   d_scores=None, stream=None):
        s, sp, n = _seeds(seeds)
        _check(LIB.pe_eval_batch(self.h, _ptr(d_genomes), pop, sp, n, vary, max_steps, _ptr(d_dist),
                                 _ptr(d_steps), _ptr(d_scores), stream))

    def evaluate_population(self, genomes, seeds, vary=0, max_steps=MAX_STEPS, want_dist=True,
                            want_steps=True, want_scores=True, out=None):
        """Host arrays in, host arrays out (genomes: float32 [pop][35])."""
        g = np.ascontiguousarray(genomes, dtype=np.float32)
        pop = g.shape[0]
        s, sp, n = _seeds(seeds)
        if out is None:
            out = {}
            if want_dist:
                out["dist"] = np.empty(pop * n, np.float32)
            if want_steps:
                out["steps"] = np.empty(pop * n, np.int32)
            if want_scores:
                out["scores"] = np.empty(pop, np.float32)
        _check(LIB.pe_evaluate_population(self.h, _ptr(g), pop, sp, n, vary, max_steps, _ptr(out.get("dist")),
                                          _ptr(out.get("steps")), _ptr(out.get("scores"))))
        return out

    def audit(self, genome, seeds, want_dist=False):
        """pe_audit: one genome under len(seeds) scenarios; the AUDIT_STATS statistics (and the
        distances when asked) as host arrays."""
        g = np.ascontiguousarray(genome, dtype=np.float32).reshape(-1)
        s, sp, n = _seeds(seeds)
        out = {"stats": np.empty(AUDIT_STATS, np.float32)}
        if want_dist:
            out["dist"] = np.empty(n, np.float32)
        _check(LIB.pe_audit(self.h, _ptr(g), sp, n, _ptr(out["stats"]), _ptr(out.get("dist"))))
        return out

    def grad(self, d_genomes, pop, seeds, d_grad, vary=0, max_steps=MAX_STEPS, checkpoint_every=60, d_obj=None,
             d_dist=None, stream=None):
        """pe_grad: d(objective)/d(genome) [pop][35] into d_grad; objective [pop] and smoothed
        distances [pop][nseeds] into d_obj / d_dist when given."""
        s, sp, n = _seeds(seeds)
        _check(LIB.pe_grad(self.h, _ptr(d_genomes), pop, sp, n, vary, max_steps, checkpoint_every, _ptr(d_obj),
                           _ptr(d_grad), _ptr(d_dist), stream))

    def objective(self, d_genomes, pop, seeds, precision=64, vary=0, max_steps=MAX_STEPS, d_obj=None, d_dist=None,
                  stream=None):
        """pe_objective: the smoothed objective [pop] / distances [pop][nseeds] (float64 device
        buffers) from a forward pass in FP32 or FP64."""
        s, sp, n = _seeds(seeds)
        _check(LIB.pe_objective(self.h, _ptr(d_genomes), pop, sp, n, vary, max_steps, precision, _ptr(d_obj),
                                _ptr(d_dist), stream))

    def evolve(self, pop, gens, nseeds, seed, max_steps=MAX_STEPS, polish_top=0, polish_steps=0, polish_lr=1e-2,
               polish_max_steps=0, holdout=128, holdout_base=100003, audit=0, audit_base=9001, history=True):
        """pe_evolve: the device GA (plain, or hybrid with polish_top > 0).  Returns (result dict,
        history [gens][5] or None: train best, holdout, mean, p90, cumulative device seconds)."""
        cfg = EvolveConfig(pop, gens, nseeds, seed, max_steps, polish_top, polish_steps, polish_lr, polish_max_steps,
                           holdout, holdout_base, audit, audit_base)
        res = EvolveResult()
        hist = np.zeros((gens, 5), np.float32) if history else None
        _check(LIB.pe_evolve(self.h, C.byref(cfg), _ptr(hist), C.byref(res)))
        out = {k: getattr(res, k) for k, _ in EvolveResult._fields_ if k != "best_genome"}
        out["best_genome"] = np.array(res.best_genome[:], np.float32)
        return out, hist

    def plane_table(self, pop, d_mp=None, d_nt=None, d_off=None, d_ext=None, d_pc=None, d_pn=None, stream=None):
        total = _I()
        _check(LIB.pe_plane_table(self.h, pop, _ptr(d_mp), _ptr(d_nt), _ptr(d_off), _ptr(d_ext), _ptr(d_pc),
                                  _ptr(d_pn), C.byref(total), stream))
        return total.value

    def autotune(self, d_genomes, pop, seeds, vary=0, max_steps=MAX_STEPS):
        s, sp, n = _seeds(seeds)
        c = Config()
        _check(LIB.pe_autotune(self.h, _ptr(d_genomes), pop, sp, n, vary, max_steps, C.byref(c)))
        return c

    def last_timing(self):
        ms = np.zeros(3, np.float32)
        n = _I()
        _check(LIB.pe_last_timing(self.h, ms.ctypes.data, C.byref(n)))
        return {"prepare_ms": float(ms[0]), "flight_ms": float(ms[1]), "scores_ms": float(ms[2]),
                "launches": n.value}

    def debug_release(self, pop, seeds, vary, d_state_out, stream=None):
        s, sp, n = _seeds(seeds)
        _check(LIB.pe_debug_release(self.h, pop, sp, n, vary, _ptr(d_state_out), stream))

    def debug_step(self, pop, seeds, vary, max_steps, d_state_in, d_state_out, d_FT, d_done, d_fit, step,
                   lanes=32, stream=None):
        s, sp, n = _seeds(seeds)
        _check(LIB.pe_debug_step(self.h, pop, sp, n, vary, max_steps, _ptr(d_state_in), _ptr(d_state_out),
                                 _ptr(d_FT), _ptr(d_done), _ptr(d_fit), step, lanes, stream))


class PanelBuf:
    """The reference's boundary: panelbuf_alloc / gpu_prepare / gpu_sim / panelbuf_free."""

    def __init__(self, pop):
        h = _VP()
        _check(LIB.pe_panelbuf_alloc(pop, C.byref(h)))
        self.h = h

    def free(self):
        if self.h:
            _check(LIB.pe_panelbuf_free(self.h))
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def prepare(self, d_genomes, pop, stream=None):
        _check(LIB.pe_prepare(_ptr(d_genomes), self.h, pop, stream))

    def sim(self, pop, seed, d_fitness, d_rec=None, rec_every=1, rec_cap=0, spread=0.0, vary=0, stream=None):
        _check(LIB.pe_sim(self.h, pop, seed, _ptr(d_fitness), _ptr(d_rec), rec_every, rec_cap, float(spread),
                          vary, stream))


def robust_scores(d_samples, pop, nseeds, d_scores, stream=None):
    _check(LIB.pe_robust_scores(_ptr(d_samples), pop, nseeds, _ptr(d_scores), stream))


# pe_distance_stats / pe_audit: min p05 p10 p25 median mean sd p75 p90 p95 max CVaR10 failures
AUDIT_STATS = 13
AUDIT_NAMES = ("min", "p05", "p10", "p25", "median", "mean", "sd", "p75", "p90", "p95", "max", "cvar10", "failures")


def distance_stats(d_dist, n, d_stats, stream=None):
    """pe_distance_stats: the audit statistics of n device distances into d_stats[13] (device)."""
    _check(LIB.pe_distance_stats(_ptr(d_dist), n, _ptr(d_stats), stream))


def station_mode(ieee):
    _check(LIB.pe_debug_station_mode(int(ieee)))


def random_genomes(seed, n):
    """Genomes drawn like the reference's grand() from std::mt19937(seed)."""
    g = np.empty((n, GENOME_FLOATS), np.float32)
    _check(LIB.pe_random_genomes(seed, n, g.ctypes.data))
    return g


def sanitize_genomes(genomes):
    """Clamp float32 genomes [n][35] to the bounds in place (the reference's sanitize()); returns them."""
    g = np.ascontiguousarray(genomes, np.float32)
    _check(LIB.pe_sanitize_genomes(g.ctypes.data, g.shape[0]))
    return g


def genome_bounds():
    lo = np.empty(GENOME_FLOATS, np.float32)
    hi = np.empty(GENOME_FLOATS, np.float32)
    _check(LIB.pe_genome_bounds(lo.ctypes.data, hi.ctypes.data))
    return lo, hi


def save_genomes(path, genomes):
    g = np.ascontiguousarray(genomes, np.float32)
    _check(LIB.pe_save_genomes(path.encode(), g.ctypes.data, g.shape[0]))


def load_genomes(path, cap=None):
    n = _I()
    _check(LIB.pe_load_genomes(path.encode(), None, 0, C.byref(n)))
    cap = n.value if cap is None else min(cap, n.value)
    g = np.empty((cap, GENOME_FLOATS), np.float32)
    _check(LIB.pe_load_genomes(path.encode(), g.ctypes.data, cap, C.byref(n)))
    return g


def save_best(path, genome):
    g = np.ascontiguousarray(genome, np.float32).reshape(GENOME_FLOATS)
    _check(LIB.pe_save_best(path.encode(), g.ctypes.data))


def load_best(path):
    g = np.empty(GENOME_FLOATS, np.float32)
    _check(LIB.pe_load_best(path.encode(), g.ctypes.data))
    return g


def fp32_peak_tflops(device=0):
    t = C.c_float()
    _check(LIB.pe_fp32_peak_probe(device, C.byref(t)))
    return float(t.value)


def topk(d_scores, n, k, d_idx, d_top=None, stream=None):
    _check(LIB.pe_topk(_ptr(d_scores), n, k, _ptr(d_idx), _ptr(d_top), stream))


def select_top(d_genomes, d_scores, pop, k, d_top, d_idx, stream=None):
    _check(LIB.pe_select_top(_ptr(d_genomes), _ptr(d_scores), pop, k, _ptr(d_top), _ptr(d_idx), stream))


def ga_step(d_genomes, d_scores, pop, gen, gens, seed, d_next, stream=None):
    _check(LIB.pe_ga_step(_ptr(d_genomes), _ptr(d_scores), pop, gen, gens, seed, _ptr(d_next), stream))


def genome_objective(engine, genomes, seeds, vary=0, max_steps=MAX_STEPS, checkpoint_every=60):
    """The smoothed tail-aware objective of each genome as a differentiable torch function.

    genomes: float32 CUDA tensor [pop, 35] -> objective [pop].  Forward and backward are one
    pe_grad call (the gradient is computed with the objective and kept for backward), so
    backward returns grad_output[:, None] * d(objective)/d(genome)."""
    import torch

    class _Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, g):
            g = g.detach().contiguous()
            pop = g.shape[0]
            obj = torch.empty(pop, device=g.device, dtype=torch.float32)
            grad = torch.empty(pop, GENOME_FLOATS, device=g.device, dtype=torch.float32)
            engine.grad(g, pop, seeds, grad, vary=vary, max_steps=max_steps, checkpoint_every=checkpoint_every,
                        d_obj=obj, stream=torch.cuda.current_stream(g.device).cuda_stream)
            ctx.save_for_backward(grad)
            return obj

        @staticmethod
        def backward(ctx, grad_out):
            (grad,) = ctx.saved_tensors
            return grad_out[:, None] * grad

    return _Objective.apply(genomes)


def eval_batch_noalloc(d_genomes, pop, seeds, vary=0, max_steps=MAX_STEPS, d_dist=None, d_steps=None,
                       d_scores=None, stream=None):
    """pe_eval_batch_noalloc: the batched evaluation on the library's static working memory."""
    s, sp, n = _seeds(seeds)
    _check(LIB.pe_eval_batch_noalloc(_ptr(d_genomes), pop, sp, n, vary, max_steps, _ptr(d_dist), _ptr(d_steps),
                                     _ptr(d_scores), stream))
