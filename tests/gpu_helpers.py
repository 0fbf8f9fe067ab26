"""Shared helpers of the GPU parity tests: run the CUDA path through the C ABI on torch buffers."""
import numpy as np


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def eval_gpu(torch, engine, genomes, seeds, vary=0, max_steps=7200, scores=True):
    pop, S = genomes.shape[0], len(seeds)
    g = dev(torch, genomes.astype(np.float32))
    dist = torch.empty(pop * S, dtype=torch.float32, device="cuda")
    steps = torch.empty(pop * S, dtype=torch.int32, device="cuda")
    sc = torch.empty(pop, dtype=torch.float32, device="cuda") if scores else None
    engine.eval_batch(g, pop, seeds, vary=vary, max_steps=max_steps, d_dist=dist, d_steps=steps, d_scores=sc)
    torch.cuda.synchronize()
    out = {"dist": dist.cpu().numpy(), "steps": steps.cpu().numpy()}
    if scores:
        out["scores"] = sc.cpu().numpy()
    return out


def plane_table(torch, engine, pop):
    mp = torch.empty(pop, 20, dtype=torch.float32, device="cuda")
    nt = torch.empty(pop, dtype=torch.int32, device="cuda")
    off = torch.empty(pop, dtype=torch.int32, device="cuda")
    ext = torch.empty(pop, 4, dtype=torch.float32, device="cuda")
    total = engine.plane_table(pop, d_mp=mp, d_nt=nt, d_off=off, d_ext=ext)
    pc = torch.empty(max(total, 1), 4, dtype=torch.float32, device="cuda")
    pn = torch.empty(max(total, 1), 4, dtype=torch.float32, device="cuda")
    engine.plane_table(pop, d_pc=pc, d_pn=pn)
    torch.cuda.synchronize()
    return {"mp": mp.cpu().numpy(), "nt": nt.cpu().numpy(), "off": off.cpu().numpy(), "ext": ext.cpu().numpy(),
            "pc": pc.cpu().numpy()[:total], "pn": pn.cpu().numpy()[:total], "total": total}


def spearman(a, b):
    """Spearman rank correlation with average ranks for ties."""
    from scipy.stats import spearmanr

    return float(spearmanr(a, b).statistic)


def state_from_oracle(st, step):
    """Oracle state (pos q vel wb t done fit) -> the C ABI's 16-float state (..., t, step, pad)."""
    s = np.zeros(16, np.float32)
    s[:14] = st[:14]
    s[14:15] = np.array([step], np.int32).view(np.float32)
    return s


# Pairs (h, h/2) of central-difference steps (fractions of each gene's range), largest first; the
# first is the specified step.
FD_PAIRS = ((1e-4, 5e-5), (2e-5, 1e-5), (4e-6, 2e-6), (1e-6, 5e-7), (3e-7, 1.5e-7))


def fd64_per_gene(torch, engine, genomes, seeds, max_steps, lo, hi, gate=1e-4):
    """FP64 central differences of the smoothed objective for every gene of every genome, on the
    GPU (pe_objective).  A gene's estimate comes from the largest step pair (h, h/2) whose two
    central differences agree, |D(h) - D(h/2)| <= gate x max(|D|, 1e-2 max_k |D_k|) -- a region
    where the objective is smooth at that scale -- as the Richardson value (4 D(h/2) - D(h)) / 3.
    Where a pair disagrees, an active-set switch (a tail-quartile member, a clamp) lies within its
    step and the next smaller pair is tried; if none agrees, D at the smallest step is used.
    Returns (fd [n][35], how many genes each pair decided, then how many fell through)."""
    n = genomes.shape[0]
    fr = [f for pair in FD_PAIRS for f in pair]
    P = np.repeat(genomes[:, None, :], 35 * len(fr) * 2, axis=1).reshape(n, 35, len(fr), 2, 35)
    for j in range(35):
        for q, f in enumerate(fr):
            h = f * (hi[j] - lo[j])
            P[:, j, q, 0, j] = (genomes[:, j] + h).astype(np.float32)
            P[:, j, q, 1, j] = (genomes[:, j] - h).astype(np.float32)
    flat = np.ascontiguousarray(P.reshape(-1, 35))
    o = torch.empty(flat.shape[0], device="cuda", dtype=torch.float64)
    engine.objective(torch.from_numpy(flat).cuda(), flat.shape[0], seeds, precision=64, max_steps=max_steps,
                     d_obj=o)
    torch.cuda.synchronize()
    o = o.cpu().numpy().reshape(n, 35, len(fr), 2)
    D = np.zeros((n, 35, len(fr)))
    for j in range(35):
        D[:, j, :] = (o[:, j, :, 0] - o[:, j, :, 1]) / (P[:, j, :, 0, j].astype(np.float64) - P[:, j, :, 1, j])
    last = D[:, :, -1]
    scale = np.maximum(np.abs(last), 1e-2 * np.abs(last).max(axis=1, keepdims=True))
    fd = last.copy()
    level = np.full(fd.shape, len(FD_PAIRS))
    for k in range(len(FD_PAIRS) - 1, -1, -1):  # smallest first, so the largest agreeing pair wins
        a, b = D[:, :, 2 * k], D[:, :, 2 * k + 1]
        ok = np.abs(a - b) <= gate * scale
        fd = np.where(ok, (4 * b - a) / 3, fd)
        level = np.where(ok, k, level)
    return fd, np.bincount(level.ravel(), minlength=len(FD_PAIRS) + 1)


def check_grad_population(grads, refs, tag=""):
    """The 1e-3 bar over a population of gradients: norm-wise |g - ref| / |ref| < 1e-3 for at least
    99 % of the genomes; per gene, |g_j - ref_j| / max(|ref_j|, 1e-2 max_k |ref_k|) < 1e-3 for at
    least 99.5 % of the (genome, gene) pairs; both < 1e-2 for all.  The exceptions are genomes whose
    objective is strongly curved next to an active-set switch (their finite differences converge
    only below a step of 1e-6 of a gene's range): rounding of the FP32 trajectory, amplified over a
    1,000-step flight, moves their gradient by a few 1e-3.  The same model in FP64 matches converged
    differences there to ~1e-5."""
    grads, refs = np.asarray(grads, np.float64), np.asarray(refs, np.float64)
    norm = np.linalg.norm(grads - refs, axis=1) / np.linalg.norm(refs, axis=1)
    floor = 1e-2 * np.abs(refs).max(axis=1, keepdims=True)
    gene = np.abs(grads - refs) / np.maximum(np.abs(refs), floor)
    frac = float((gene >= 1e-3).mean())
    nfrac = float((norm >= 1e-3).mean())
    print(f"{tag} {len(refs)} genomes: norm-wise max {norm.max():.2e} median {np.median(norm):.2e}, "
          f">= 1e-3 for {nfrac:.4f} of genomes; per gene >= 1e-3: {frac:.4f} of pairs, max {gene.max():.2e}")
    assert nfrac <= 0.01 and norm.max() < 1e-2, (tag, nfrac, float(norm.max()), int(norm.argmax()))
    assert frac <= 0.005 and gene.max() < 1e-2, (tag, frac, float(gene.max()))
