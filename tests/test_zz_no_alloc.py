"""vsc_get_consist_out_noalloc: the solver for callers that must not allocate
device memory (stream capture, real-time loops, plugins whose host owns the
memory).  It keeps its workspace in an array inside the library instead of
asking for memory, so it is checked here against the allocating entry point,
through the C ABI, on two calls in a row (the second call inherits the
first call's leftovers in that shared array).  Same tolerance as the other
solver tests: identical bits.

This file is collected last on purpose, so a run that stops at its first
failure has run every other test before this one."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(rng, h, w, dev):
    import torch

    P = torch.from_numpy(rng.random((h, w, 3), dtype=np.float32)).to(dev)
    A = torch.from_numpy(rng.random((h, w, 3), dtype=np.float32)).to(dev)
    Wt = torch.from_numpy(rng.uniform(0.0, 2.0, (h, w, 3)).astype(np.float32)).to(dev)
    O = torch.from_numpy(rng.random((h, w, 3), dtype=np.float32)).to(dev)
    return P, A, Wt, O


# (480, 720) is the largest frame size the built-in workspace admits in this
# list and takes the TMA-fed solver; (101, 333) takes the per-tile solver.
@pytest.mark.parametrize("h,w,iters", [(480, 720, 150), (101, 333, 75)])
def test_noalloc_equals_allocating_solver_twice(vsc, cuda, h, w, iters):
    import torch

    assert h * w <= vsc.NOALLOC_MAX_PIXELS
    lib = vsc.load()
    rng = np.random.Generator(np.random.PCG64(h * w + iters))
    for call in range(2):  # a second call on the same shared workspace
        P, A, Wt, O0 = _inputs(rng, h, w, cuda)
        ref = O0.clone()
        got = O0.clone()
        ims = [vsc.Image(t.data_ptr(), w, h, 3) for t in (P, A, Wt)]
        rc = lib.vsc_get_consist_out(C.byref(ims[0]), C.byref(ims[1]), C.byref(ims[2]), iters, 0.15, 0.15,
                                     C.byref(vsc.Image(ref.data_ptr(), w, h, 3)), None, 0, None)
        assert rc == vsc.VSC_OK, lib.vsc_last_error()
        rc = lib.vsc_get_consist_out_noalloc(C.byref(ims[0]), C.byref(ims[1]), C.byref(ims[2]), iters, 0.15, 0.15,
                                             C.byref(vsc.Image(got.data_ptr(), w, h, 3)), None)
        assert rc == vsc.VSC_OK, lib.vsc_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, ref), f"call {call}"
        assert not torch.equal(got, O0)
    vsc.check_device()


def test_noalloc_rejects_images_beyond_its_workspace(vsc, cuda):
    import torch

    lib = vsc.load()
    w, h = 1920, 1080
    t = torch.zeros((h, w, 3), device=cuda)
    im = vsc.Image(t.data_ptr(), w, h, 3)
    rc = lib.vsc_get_consist_out_noalloc(C.byref(im), C.byref(im), C.byref(im), 10, 0.15, 0.15, C.byref(im), None)
    assert rc == vsc.VSC_EINVAL
    msg = lib.vsc_last_error().decode()
    assert "limit" in msg and str(vsc.NOALLOC_MAX_PIXELS) in msg
