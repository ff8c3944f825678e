"""Train the learned flow upsampler (vsc_upsampler_*) for the FLOWDOWNSCALE=2
fast mode, on synthetic frame pairs whose flows the library's own estimator
computes: the input is the flow estimated on the frames resized to half size
(nearest, as the stabilizer's fast mode does) plus the full-size luma, the
target the flow estimated at full size.

    python video-stream-consistency_gb300/train_upsampler.py [--pairs 2000] [--out weights.npz]

Pairs come from seeded synthetic streams (Gaussian blobs advected by a
smooth flow, re-drawn every 30 frames), 1920x1080 by default; random 64x64
crops of (input, target) feed Adam with an L1 loss.  Held-out pairs measure
the end-point error against the full-size flow, learned (with the 0.5 px
fallback) versus bilinear.  Writes the parameters and the run's figures to
an .npz and a .json beside it.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _pkg():
    if "vsc_gb300" in sys.modules:
        return sys.modules["vsc_gb300"]
    spec = importlib.util.spec_from_file_location("vsc_gb300", HERE / "__init__.py", submodule_search_locations=[str(HERE)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["vsc_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def nearest(img, ow, oh):
    """The stabilizer's downscaling (QImage::scaled, fast): source pixel under each target centre."""
    import torch

    h, w = img.shape[:2]
    xs = torch.clamp(((2 * torch.arange(ow, device=img.device) + 1) * w) // (2 * ow), max=w - 1)
    ys = torch.clamp(((2 * torch.arange(oh, device=img.device) + 1) * h) // (2 * oh), max=h - 1)
    return img[ys][:, xs].contiguous()


def make_pairs(vsc, n_pairs, w, h, seed, device):
    """(input, target) per pair: input (h, w, 3) base flow + luma, target (h, w, 2)."""
    import torch

    from vsc_gb300 import synth

    fw, fh = int(round(w / 2)), int(round(h / 2))
    out = []
    per_stream = 25
    for k in range((n_pairs + per_stream - 1) // per_stream):
        s = synth.SyntheticStream(w, h, seed=seed + k, device=device)
        frames = [s.frame(t) for t in range(per_stream + 1)]
        imgs = [vsc.char_to_float_image(torch.from_numpy(o).to(device)) for o, _ in frames]
        for t in range(per_stream):
            if len(out) == n_pairs:
                break
            a, b = imgs[t], imgs[t + 1]
            full, _ = vsc.flow_estimate(a, b)
            small, _ = vsc.flow_estimate(nearest(a, fw, fh), nearest(b, fw, fh))
            inp = vsc.Upsampler.prepare(small, a)
            out.append((inp, full[..., :2].contiguous(), small, a))
    return out


def epe(flow, target):
    import torch

    return float(torch.sqrt(((flow[..., :2] - target) ** 2).sum(-1)).mean())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--held-out", type=int, default=50)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--crop", type=int, default=64)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=str(HERE / "upsampler_weights.npz"))
    args = ap.parse_args()

    import torch

    vsc = _pkg()
    vsc.build()
    vsc.load()
    dev = "cuda"
    t0 = time.time()
    # training pairs: only crops are kept (1080p pairs would not all fit in memory)
    g = torch.Generator().manual_seed(args.seed)
    crops_in, crops_t = [], []
    remaining = args.pairs
    chunk = 100
    k = 0
    while remaining > 0:
        n = min(chunk, remaining)
        for inp, tgt, _, _ in make_pairs(vsc, n, args.width, args.height, args.seed + 1000 * k, dev):
            for _ in range(4):
                y = int(torch.randint(0, args.height - args.crop + 1, (1,), generator=g))
                x = int(torch.randint(0, args.width - args.crop + 1, (1,), generator=g))
                crops_in.append(inp[y:y + args.crop, x:x + args.crop].clone())
                crops_t.append(tgt[y:y + args.crop, x:x + args.crop].clone())
        remaining -= n
        k += 1
    crops_in = torch.stack(crops_in)
    crops_t = torch.stack(crops_t)
    t_data = time.time() - t0

    up = vsc.Upsampler()
    losses = []
    t1 = time.time()
    for step in range(args.steps):
        idx = torch.randint(0, crops_in.shape[0], (args.batch,), generator=g).to(dev)
        lr = args.lr * 0.5 * (1 + np.cos(np.pi * step / args.steps))  # cosine decay
        loss = up.train_step(crops_in[idx].contiguous(), crops_t[idx].contiguous(), lr)
        if step % 100 == 0 or step == args.steps - 1:
            losses.append((step, loss))
    torch.cuda.synchronize()
    t_train = time.time() - t1

    # held-out pairs (other seeds): end-point error against the full-size flow
    res = {"bilinear": [], "learned": []}
    for inp, tgt, small, frame in make_pairs(vsc, args.held_out, args.width, args.height, args.seed + 999_999, dev):
        res["bilinear"].append(epe(inp, tgt))
        res["learned"].append(epe(up.apply(small, frame), tgt))
    params = up.params()
    meta = {
        "pairs": args.pairs, "crops": int(crops_in.shape[0]), "crop": args.crop, "steps": args.steps,
        "batch": args.batch, "lr": args.lr, "seed": args.seed, "size": [args.width, args.height],
        "loss_first_last": [losses[0][1], losses[-1][1]], "loss_curve": losses,
        "held_out_pairs": args.held_out,
        "epe_bilinear_px": float(np.mean(res["bilinear"])), "epe_learned_px": float(np.mean(res["learned"])),
        "seconds_data": t_data, "seconds_train": t_train, "param_count": int(params.size),
    }
    np.savez(args.out, params=params)
    Path(args.out).with_suffix(".json").write_text(json.dumps(meta, indent=1))
    print(json.dumps({k: v for k, v in meta.items() if k != "loss_curve"}))


if __name__ == "__main__":
    main()
