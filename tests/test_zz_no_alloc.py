"""bm_refine_noalloc: the refinement stage for callers that cannot allocate device
memory while they run (pipelines that allocate only at start-up, plugin hosts that
own the memory budget, real-time threads that must not take the synchronisation
of cudaMalloc).  It keeps its intermediate planes in a fixed array inside the
library.  This test calls it through the C ABI twice in a row, with different
inputs, and checks each result against the context path (bm_process) within the
refined-flow tolerance of the other parity tests, once more at 2048x1024, where the
four scratch planes fill the array to its last element, and checks the size limit
and the rejection of outputs that overlap inputs and of unusable sigmas.

The file name sorts last so that a run stopping at the first failure has already
run every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import briefmatch_gb300 as bm

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

FLOW_TOL = 1e-4  # px, as for every refined-flow comparison


def _inputs(seed, W, H):
    rng = np.random.default_rng(seed)
    U = (rng.normal(0, 3, size=(H, W)) + np.linspace(-6, 6, W)[None, :]).astype(np.float32)
    V = (rng.normal(0, 3, size=(H, W)) + np.linspace(4, -4, H)[:, None]).astype(np.float32)
    from briefmatch_gb300 import synth

    I = synth.make_frame(rng, W, H, blobs=10).astype(np.float32)
    return U, V, I


def _context_path(prm, U, V, I):
    eng = bm.BriefMatch(prm)
    eng.setup()
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.write_buffer(bm.BM_BUF_FLOW_IN, np.concatenate([U.ravel(), V.ravel()]))
    d_I = torch.from_numpy(I).cuda()
    eng.process(d_I.data_ptr())
    torch.cuda.synchronize()
    out = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, *U.shape)
    eng.clean()
    return out


def test_refine_noalloc_matches_context_path_twice():
    W, H = 160, 96
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=32)
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (1, 2):
        U, V, I = _inputs(seed, W, H)
        want = _context_path(prm, U, V, I)
        dU, dV, dI = (torch.from_numpy(a).cuda() for a in (U, V, I))
        oU = torch.full((H, W), float("nan"), device="cuda")
        oV = torch.full((H, W), float("nan"), device="cuda")
        bm.refine_noalloc(dU.data_ptr(), dV.data_ptr(), dI.data_ptr(), oU.data_ptr(), oV.data_ptr(), W, H,
                          prm.fsize, prm.sEPE, prm.sI, prm.sS, stream)
        torch.cuda.synchronize()
        got = np.stack([oU.cpu().numpy(), oV.cpu().numpy()])
        assert np.isfinite(got).all()
        err = float(np.abs(got - want).max())
        assert err <= FLOW_TOL, (seed, err)


def test_refine_noalloc_rejects_oversize():
    L = bm.lib()
    maxpx = L.bm_refine_noalloc_max_pixels()
    assert maxpx == 2 * 1024 * 1024
    dummy = torch.zeros(4, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    st = L.bm_refine_noalloc(p, p, p, p, p, 4096, 1024, 13, 0.4, 0.1, 9.0, None)
    assert st == bm.BM_ERR_LIMIT
    assert "fixed scratch" in L.bm_last_error().decode()


def test_refine_noalloc_at_the_scratch_limit():
    """2048 x 1024 = the largest frame: the fourth scratch plane ends at the array's
    last element."""
    W, H = 2048, 1024
    assert W * H == bm.lib().bm_refine_noalloc_max_pixels()
    prm = bm.BMParams.derive(W, H, 1.0, 1.0, N=32)
    U, V, I = _inputs(3, W, H)
    want = _context_path(prm, U, V, I)
    dU, dV, dI = (torch.from_numpy(a).cuda() for a in (U, V, I))
    oU = torch.full((H, W), float("nan"), device="cuda")
    oV = torch.full((H, W), float("nan"), device="cuda")
    bm.refine_noalloc(dU.data_ptr(), dV.data_ptr(), dI.data_ptr(), oU.data_ptr(), oV.data_ptr(), W, H,
                      prm.fsize, prm.sEPE, prm.sI, prm.sS, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = np.stack([oU.cpu().numpy(), oV.cpu().numpy()])
    assert np.isfinite(got).all()
    err = float(np.abs(got - want).max())
    assert err <= FLOW_TOL, err


def test_refine_noalloc_rejects_aliasing_and_bad_sigmas():
    L = bm.lib()
    W, H = 64, 32
    buf = torch.zeros(6, H * W, device="cuda")
    p = [ctypes.c_void_p(buf[k].data_ptr()) for k in range(6)]
    half = ctypes.c_void_p(buf[0].data_ptr() + 4 * (H * W // 2))   # overlaps plane 0 and plane 1
    for uo, vo in ((p[0], p[4]), (p[3], p[1]), (p[4], p[2]), (half, p[4]), (p[4], p[4])):
        st = L.bm_refine_noalloc(p[0], p[1], p[2], uo, vo, W, H, 5, 0.4, 0.1, 2.0, None)
        assert st == bm.BM_ERR_INVALID
        assert "overlap" in L.bm_last_error().decode()
    for sE, sI_, sS in ((float("inf"), 0.1, 2.0), (0.4, float("nan"), 2.0), (0.4, 0.1, 0.0), (0.4, 0.1, -1.0)):
        st = L.bm_refine_noalloc(p[0], p[1], p[2], p[3], p[4], W, H, 5, sE, sI_, sS, None)
        assert st == bm.BM_ERR_INVALID
    st = L.bm_refine_noalloc(p[0], p[1], p[2], p[3], p[4], W, H, 5, 0.4, 0.1, 1e6, None)
    assert st == bm.BM_ERR_LIMIT
    # still usable
    st = L.bm_refine_noalloc(p[0], p[1], p[2], p[3], p[4], W, H, 5, 0.4, 0.1, 2.0, None)
    assert st == bm.BM_OK
    torch.cuda.synchronize()
