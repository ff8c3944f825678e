"""The reference's frame loop over the CPU restatement (test helper, not a
test module): the comparator of the whole-stream GPU tests."""
from __future__ import annotations

import numpy as np


def run_oracle_stream(oracle, frames, flows=None, hp=None, downscale=1, occlusion=False, solver_form="exact"):
    """The reference's driver loop (stabilizefiles.cpp:108-131 with
    videostabilizer.cpp:136-265) over the restatement."""
    orig = [oracle.rgba_to_float(o) for o, _ in frames]
    proc = [oracle.rgba_to_float(p) for _, p in frames]
    h, w = orig[0].shape[:2]
    last = proc[2]
    outs = []
    for t in range(1, len(frames) - 1):
        if flows is not None:
            ff, fb = flows[t]
        elif downscale > 1:
            # videostabilizer.cpp:93-94: C round(), halves away from zero
            fw, fh = int(np.floor(np.float32(w) / np.float32(downscale) + 0.5)), int(
                np.floor(np.float32(h) / np.float32(downscale) + 0.5))
            small = [nearest(orig[t], fw, fh), nearest(orig[t + 1], fw, fh)]
            ff = oracle.bilinear(oracle.flow_estimate(small[0], small[1]), w, h)
            fb = oracle.bilinear(oracle.flow_estimate(small[1], small[0]), w, h)
        else:
            ff = oracle.flow_estimate(orig[t], orig[t + 1])
            fb = oracle.flow_estimate(orig[t + 1], orig[t])
        out, rgba = oracle.stab_pass(orig[t - 1:t + 2], proc[t - 1:t + 2], ff, fb, last, hp, occlusion_mask=occlusion,
                                     solver_form=solver_form)
        outs.append((out, rgba, ff, fb))
        last = out
    return outs


def nearest(img, ow, oh):
    h, w = img.shape[:2]
    xs = np.minimum(w - 1, ((2 * np.arange(ow) + 1) * w) // (2 * ow))
    ys = np.minimum(h - 1, ((2 * np.arange(oh) + 1) * h) // (2 * oh))
    return np.ascontiguousarray(img[ys][:, xs])
