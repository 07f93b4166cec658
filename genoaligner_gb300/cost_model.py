"""The learned cost model: training, labels, checkpoints.

The network (learned.cu) maps a pair's 66 sketch features to
[log2(d + 1), log2((d + 1)^2 + 1)] -- the edit distance and the WFA's
wavefront-cell work.  It is trained on the GPU by the library's own forward,
backward and Adam kernels, on pairs labelled by the library's exact WFA
(score-only at smax 250 for the short pairs and 2048 for the long ones, pairs
unresolved there left out, so every training label is the true distance):
2,000,000 pairs of the mixed-divergence distribution (150-250 bp) and 20,000
pairs of the long distribution (1-10 kb, error 1-15 %, geometric indels)
repeated 10 times in the training set; 10 epochs, batch 8192, the rate
2e-3 x 0.75 per epoch (--short-only: the short pairs alone).

Checkpoint: an .npz with the fp32 parameters, a format version and the
training seed; ``load_default()`` puts the committed model
(models/wfa_cost_v1.npz) on the current device.  Routing never changes a
result, so a missing or poor model only costs time.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import api, workloads

FORMAT_VERSION = 1
DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "wfa_cost_v1.npz")
LABEL_SMAX = 250
LABEL_SMAX_LONG = 2048
LONG_REPEAT = 10
EPOCHS = 10
DECAY = 0.75


def training_pairs(n: int = 2_000_000, seed: int = 1001) -> workloads.PairSet:
    """Pairs of the mixed-divergence distribution, separately seeded."""
    return workloads.wfa_mixed(n=n, seed=seed)


def training_pairs_long(n: int = 20_000, seed: int = 1002) -> workloads.PairSet:
    """Pairs of the long distribution (1-10 kb), separately seeded."""
    return workloads.wfa_long_1k_10k(n=n, seed=seed)


def labels_and_features(ps: workloads.PairSet, chunk: int = 250_000, label_smax: int = LABEL_SMAX):
    """Exact distances (GPU WFA, score-only, at label_smax) and sketch
    features, as torch tensors on the current device: (features [n,66],
    targets [n,2], distance [n], lower bound [n])."""
    import torch
    feats, targs, dists, lbs = [], [], [], []
    for lo in range(0, ps.n, chunk):
        sub = ps if (lo == 0 and ps.n <= chunk) else _slice(ps, lo, min(ps.n, lo + chunk))
        b = api.DeviceBatchT(sub.a_buf, sub.a_off, sub.a_len, sub.b_buf, sub.b_off, sub.b_len)
        score = torch.empty(b.n, dtype=torch.int32, device="cuda")
        api.wfa_device(b, label_smax, False, score, None, None)
        f, lb = api.wfa_features(b)
        d = score.to(torch.float32)
        t = torch.stack([torch.log2(d + 1), torch.log2((d + 1) ** 2 + 1)], dim=1)
        keep = score >= 0
        feats.append(f[keep]); targs.append(t[keep]); dists.append(score[keep]); lbs.append(lb[keep])
    return torch.cat(feats), torch.cat(targs).contiguous(), torch.cat(dists), torch.cat(lbs)


def _slice(ps: workloads.PairSet, lo: int, hi: int) -> workloads.PairSet:
    a0, a1 = int(ps.a_off[lo]), int(ps.a_off[hi - 1] + ps.a_len[hi - 1])
    b0, b1 = int(ps.b_off[lo]), int(ps.b_off[hi - 1] + ps.b_len[hi - 1])
    return workloads.PairSet(ps.name, ps.a_buf[a0:a1], ps.a_off[lo:hi] - a0, ps.a_len[lo:hi],
                             ps.b_buf[b0:b1], ps.b_off[lo:hi] - b0, ps.b_len[lo:hi], ps.meta)


def train(feat, target, epochs: int = 3, batch: int = 8192, lr: float = 2e-3, seed: int = 1001,
          log=None, decay: float = 0.3) -> dict:
    """Adam on the library's kernels (the calling thread's selected model
    slot), the rate times `decay` each epoch; returns the training record."""
    import torch
    api.cost_model_set(api.cost_model_init(seed))
    n = int(feat.shape[0])
    g = torch.Generator(device="cuda").manual_seed(seed)
    losses = []
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=g)
        step_lr = lr * (decay ** ep)
        for lo in range(0, n - batch + 1, batch):
            idx = perm[lo:lo + batch]
            xb = feat[idx].contiguous()
            yb = target[idx].contiguous()
            losses.append(api.mlp_train_step(xb, yb, step_lr))
        if log:
            log(f"epoch {ep}: loss {np.mean(losses[-50:]):.4f}")
    return {"losses": losses, "seconds": time.time() - t0, "steps": len(losses), "epochs": epochs,
            "batch": batch, "lr": lr, "seed": seed}


def save(path: str, params: np.ndarray, seed: int, record: dict | None = None):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=params.astype(np.float32), version=np.int32(FORMAT_VERSION), seed=np.int64(seed),
             final_loss=np.float32(np.mean(record["losses"][-50:]) if record else np.nan))


def load(path: str = DEFAULT_PATH) -> np.ndarray:
    z = np.load(path)
    if int(z["version"]) != FORMAT_VERSION:
        raise ValueError(f"{path}: cost-model format {int(z['version'])}, expected {FORMAT_VERSION}")
    p = z["params"]
    if p.shape[0] != api.cost_model_nparams():
        raise ValueError(f"{path}: {p.shape[0]} parameters, expected {api.cost_model_nparams()}")
    return p


def load_default(path: str | None = None) -> bool:
    """Put the committed model (or the one at `path`) on the current device;
    False when absent."""
    path = path or DEFAULT_PATH
    if not os.path.exists(path):
        return False
    api.cost_model_set(load(path))
    return True


def evaluate(feat, dist, lb) -> dict:
    """Prediction quality of the loaded model against the lower-bound-only rule."""
    import torch
    y = api.mlp_forward_fast(feat)              # the pass routing uses
    pred = torch.clamp(torch.exp2(torch.clamp(y[:, 0], min=0)) - 1, min=0)
    d = dist.to(torch.float32)
    first = torch.maximum(torch.ceil(pred * 1.25 + 2), lb.to(torch.float32))
    return {
        "mae_distance": float((pred - d).abs().mean()),
        "mae_distance_lower_bound_only": float((lb.to(torch.float32) - d).abs().mean()),
        "escalation_rate": float((first < d).to(torch.float32).mean()),
        "escalation_rate_lower_bound_only": float((torch.clamp(lb.to(torch.float32), min=1) < d).to(torch.float32).mean()),
        "pairs": int(d.shape[0]),
    }


def main():
    """Train a model (GPU) by the committed model's recipe (seed 1001);
    --short-only leaves the long pairs out.  Usage: python -m
    genoaligner_gb300.cost_model [out.npz] [--short-only]"""
    import json
    import sys
    import torch
    api.load()
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    t0 = time.time()
    ps = training_pairs()
    feat, targ, dist, lb = labels_and_features(ps)
    if "--short-only" not in sys.argv[1:]:
        lf, lt, _, _ = labels_and_features(training_pairs_long(), chunk=5000, label_smax=LABEL_SMAX_LONG)
        feat = torch.cat([feat] + [lf] * LONG_REPEAT)
        targ = torch.cat([targ] + [lt] * LONG_REPEAT).contiguous()
    t1 = time.time()
    rec = train(feat, targ, epochs=EPOCHS, decay=DECAY, log=lambda s: print(s, flush=True))
    params = api.cost_model_get()
    out = args[0] if args else DEFAULT_PATH
    save(out, params, 1001, rec)
    hold = workloads.wfa_mixed(n=200_000, seed=4040)
    hf, _, hd, hl = labels_and_features(hold)
    ev = evaluate(hf, hd, hl)
    lh = workloads.wfa_long_1k_10k(n=2_000, seed=4041)
    lhf, _, lhd, lhl = labels_and_features(lh, chunk=5000, label_smax=LABEL_SMAX_LONG)
    ev_long = evaluate(lhf, lhd, lhl)
    print(json.dumps({"label_seconds": t1 - t0, "train_seconds": rec["seconds"], "steps": rec["steps"],
                      "final_loss": float(np.mean(rec["losses"][-50:])), "holdout": ev, "holdout_long": ev_long,
                      "path": out}))


if __name__ == "__main__":
    main()
