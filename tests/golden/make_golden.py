"""Generate the golden fixtures in this directory.

Run in a checkout where the reference tree is available; the
reference's own CPU custom ops (correlation.cc, warp.cc) are compiled in place
by oracle/Makefile ("make ref") and called through oracle/oracle.py:

    python tests/golden/make_golden.py

Fixtures (npz, small seeded inputs):
  ref_ops.npz   inputs and outputs of the reference CPU ops:
                Correlation (legacy 0, max_displacement 1..4, float32 and
                float64, ragged shapes) and Warp (float32 and float64; the
                input/flow distributions of the reference's own op test,
                model-conversion/test.py:139-190, at reduced size).
  stab.npz      inputs and outputs of the project's CPU restatement of the
                stabilization pass and flow estimator (no CPU code exists in
                the reference for these); pins the restatement across
                machines and compilers.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def ref_ops():
    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("reference ops not built (reference tree missing)")
    rng = np.random.Generator(np.random.PCG64(20240501))
    d = {}
    corr_cases = [(1, 8, 12, 20, 4), (2, 5, 7, 9, 4), (1, 16, 5, 33, 3), (1, 3, 6, 6, 2), (1, 4, 9, 11, 1)]
    for i, (n, c, h, w, md) in enumerate(corr_cases):
        f1 = rng.standard_normal((n, c, h, w)).astype(np.float32)
        f2 = rng.standard_normal((n, c, h, w)).astype(np.float32)
        d[f"corr{i}_f1"], d[f"corr{i}_f2"] = f1, f2
        d[f"corr{i}_md"] = np.int64(md)
        d[f"corr{i}_out"] = O.ref_correlation(f1, f2, md)
        d[f"corr{i}_out64"] = O.ref_correlation(f1.astype(np.float64), f2.astype(np.float64), md)
    # the reference's op test draws torch.rand(...)*10 features and rand flows
    warp_cases = [((2, 6, 16, 12), 1.0), ((1, 4, 11, 13), 3.0), ((1, 3, 8, 8), 9.0)]
    for i, (shape, fscale) in enumerate(warp_cases):
        x = (rng.random(shape) * 10).astype(np.float32)
        flow = (rng.random((shape[0], 2) + shape[2:]) * fscale - (0 if i == 0 else fscale / 2)).astype(np.float32)
        d[f"warp{i}_x"], d[f"warp{i}_flow"] = x, flow
        d[f"warp{i}_out"] = O.ref_warp(x, flow)
        d[f"warp{i}_out64"] = O.ref_warp(x.astype(np.float64), flow.astype(np.float64))
    np.savez_compressed(OUT / "ref_ops.npz", **d)


def stab():
    sys.path.insert(0, str(ROOT))
    import importlib.util

    pkg = ROOT / "video-stream-consistency_gb300"
    spec = importlib.util.spec_from_file_location("vsc_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["vsc_gb300"] = mod
    spec.loader.exec_module(mod)
    from vsc_gb300 import synth

    s = synth.SyntheticStream(96, 64, seed=7)
    d = {}
    orig = [s.frame(i)[0] for i in range(3)]
    proc = [s.frame(i)[1] for i in range(3)]
    d["orig_rgba"] = np.stack(orig)
    d["proc_rgba"] = np.stack(proc)
    of = [O.rgba_to_float(a) for a in orig]
    pf = [O.rgba_to_float(a) for a in proc]
    ffwd = O.flow_estimate(of[1], of[2])
    fbwd = O.flow_estimate(of[2], of[1])
    d["flow_fwd"], d["flow_bwd"] = ffwd, fbwd
    out, rgba = O.stab_pass(of, pf, ffwd, fbwd, pf[2])
    d["stab_out"], d["stab_rgba"] = out, rgba
    np.savez_compressed(OUT / "stab.npz", **d)


if __name__ == "__main__":
    ref_ops()
    stab()
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size, "bytes")
