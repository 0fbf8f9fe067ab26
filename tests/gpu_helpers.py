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
