"""The SW variant model: the cost model's network trained on Smith-Waterman labels.

Same network and kernels as the WFA cost model (learned.cu: 66 -> 128 -> 128
-> 2, bf16 weights, fp32 accumulation, the library's own forward, backward
and Adam kernels), held in model slot 1.  Inputs: the 3-mer sketch of a pair
(text with its flanks against the pattern; count differences / 64, lengths /
8192).  Outputs: the pair's best local score as a fraction of its all-match
score match * min(m, n), and log2(cells) / 32.  Labels come from the
library's exact score-only SW.

What it decides (ga_sw_device_ex / the SW extension entry with learned = 1):
which pure-ACGT pairs beyond the proven 16-bit bound try the two-pairs-per-warp
16-bit kernel.  A pair whose best reaches the 16-bit limit there is recomputed
by the 32-bit kernel, so the choice never changes a result; a wrong prediction
costs either a hand-over (predicted too low) or the slower 32-bit kernel
(predicted too high).
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import api, cost_model, workloads

FORMAT_VERSION = 1
DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "sw_variant_v1.npz")
SCORING = (2, -3, 3, 1)
SLOT = 1


def training_pairs(n: int = 12_288, seed: int = 2001) -> workloads.PairSet:
    """Pairs shaped like the long SW batch -- query log-uniform 500 bp-30 kb,
    0-5 kb random flanks each side -- with the divergence drawn per pair from
    U[2 %, 20 %] (sub/ins/del 50/25/25), separately seeded."""
    rng = np.random.default_rng(seed)
    qlen = np.rint(np.exp(rng.uniform(np.log(500), np.log(30000), size=n))).astype(np.int64)
    q = workloads.random_bases(rng, int(qlen.sum()))
    rate = rng.uniform(0.02, 0.20, size=n)
    core, core_len = workloads.mutate_point(rng, q, qlen, rate, (0.5, 0.25, 0.25))
    core_off = np.zeros(n, np.int64)
    core_off[1:] = np.cumsum(core_len)[:-1]
    lf = rng.integers(0, 5001, size=n)
    rf = rng.integers(0, 5001, size=n)
    ts = [np.concatenate([workloads.random_bases(rng, int(lf[i])), core[core_off[i]:core_off[i] + core_len[i]],
                          workloads.random_bases(rng, int(rf[i]))]) for i in range(n)]
    tlen = np.array([x.shape[0] for x in ts], np.int64)
    return workloads._pairs("sw_variant_train", np.concatenate(ts), tlen, q, qlen,
                            {"scoring": SCORING, "rate": rate})


def labels_and_features(ps: workloads.PairSet, scoring=SCORING):
    """(features [n,66], targets [n,2], scores [n]) as torch tensors on the
    current device; scores by the library's score-only SW."""
    import torch
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    score = torch.empty(b.n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * b.n, dtype=torch.int32, device="cuda")
    api.sw_device(b, scoring, False, score, pos, None, None)
    feat = api.sw_features(b)
    m = b.a_len.to(torch.float32)
    n = b.b_len.to(torch.float32)
    allm = scoring[0] * torch.minimum(m, n).clamp(min=1)
    frac = score.to(torch.float32) / allm
    t = torch.stack([frac, torch.log2(m * n + 1) / 32.0], dim=1).contiguous()
    return feat, t, score


def train(feat, target, epochs: int = 40, batch: int = 512, lr: float = 2e-3, seed: int = 2001, log=None):
    with api.model_slot(SLOT):
        return cost_model.train(feat, target, epochs=epochs, batch=batch, lr=lr, seed=seed, log=log, decay=0.92)


def save(path: str, params: np.ndarray, seed: int, record: dict | None = None):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=params.astype(np.float32), version=np.int32(FORMAT_VERSION), seed=np.int64(seed),
             final_loss=np.float32(np.mean(record["losses"][-50:]) if record else np.nan))


def load_default() -> bool:
    """Put the committed SW variant model into slot 1 of the current device;
    False when absent."""
    if not os.path.exists(DEFAULT_PATH):
        return False
    z = np.load(DEFAULT_PATH)
    if int(z["version"]) != FORMAT_VERSION or z["params"].shape[0] != api.cost_model_nparams():
        raise ValueError(f"{DEFAULT_PATH}: not a version-{FORMAT_VERSION} SW variant model")
    with api.model_slot(SLOT):
        api.cost_model_set(z["params"])
    return True


def routing_quality(ps: workloads.PairSet, scoring=SCORING) -> dict:
    """How the loaded model's 16-bit choices (sw_route_kernel's rule) compare
    with the exact outcome, beside the proven bound alone (which takes only
    pairs whose all-match score fits): pairs taken, pairs that fit 16 bits
    and were left out, pairs taken that would be handed over."""
    import torch
    feat, _, score = labels_and_features(ps, scoring)
    with api.model_slot(SLOT):
        y = api.mlp_forward_fast(feat)
    m = torch.from_numpy(ps.a_len.astype(np.float32)).cuda()
    n = torch.from_numpy(ps.b_len.astype(np.float32)).cuda()
    allm = scoring[0] * torch.minimum(m, n)
    go = scoring[2]
    pred = y[:, 0].clamp(0, 1) * allm * 1.15 + 8 * scoring[0]
    taken = pred + (1024 + go) < 32000
    bound = allm + (1024 + go) < 32000
    fits = score.to(torch.float32) < (32000 - 1024 - scoring[0])
    return {"pairs": int(m.shape[0]), "fit_16bit": int(fits.sum()),
            "taken_by_model": int(taken.sum()), "taken_by_bound": int(bound.sum()),
            "fit_but_left_by_model": int((fits & ~taken).sum()), "fit_but_left_by_bound": int((fits & ~bound).sum()),
            "taken_but_handed_over_by_model": int((taken & ~fits).sum()),
            "mae_fraction": float((y[:, 0] - score.to(torch.float32) / allm.clamp(min=1)).abs().mean())}


def main():
    """Train the default SW variant model (GPU) and print its routing quality
    on a separately seeded holdout and on the long SW batch itself."""
    import json
    import sys
    api.load()
    t0 = time.time()
    ps = training_pairs()
    feat, targ, _ = labels_and_features(ps)
    t1 = time.time()
    rec = train(feat, targ, log=lambda s: print(s, flush=True))
    with api.model_slot(SLOT):
        params = api.cost_model_get()
    out = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_PATH
    save(out, params, 2001, rec)
    hold = training_pairs(n=2048, seed=2002)
    print(json.dumps({"label_seconds": t1 - t0, "train_seconds": rec["seconds"], "steps": rec["steps"],
                      "final_loss": float(np.mean(rec["losses"][-50:])), "path": out,
                      "holdout": routing_quality(hold), "sw_long_4k": routing_quality(workloads.sw_long_4k())}))


if __name__ == "__main__":
    main()
