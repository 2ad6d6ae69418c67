"""Pipelined frames (bm_set_pipelined): each pair's refinement and output copies run
on a second stream while the next frame is matched.  The flows must be bit-identical
to the plain frame loop -- device and page-locked host outputs, with and without the
learned proposal, and across switching the mode off mid-sequence."""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

from briefmatch_gb300 import learn, synth  # noqa: E402

W, H = 120, 80


def _frames(n=7):
    frames, _ = synth.make_sequence(31, W, H, n, vmax=6.0)
    d = [torch.from_numpy(f).cuda() for f in frames]
    torch.cuda.synchronize()
    return frames, d


def _run(d, pipelined, net=None, host=False, switch_off_at=None, side=True):
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    eng = bm.BriefMatch(prm)
    eng.setup()
    if net is not None:
        bm.set_proposal(eng, net, 0.5, 1, 8)
        bm.set_proposal_stream(eng, side)
    eng.set_pipelined(pipelined)
    n = len(d) - 1
    if host:
        u = torch.empty(n, H, W).pin_memory()
        v = torch.empty(n, H, W).pin_memory()
    else:
        u = torch.empty(n, H, W, device="cuda")
        v = torch.empty(n, H, W, device="cuda")
    eng.frame(d[0].data_ptr(), True)
    for k in range(1, n + 1):
        if switch_off_at == k:
            eng.set_pipelined(False)
        eng.frame(d[k].data_ptr(), True, u[k - 1].data_ptr(), v[k - 1].data_ptr(), not host)
    eng.synchronize()
    last = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, H, W)
    eng.clean()
    return u.cpu().numpy(), v.cpu().numpy(), last


@pytest.mark.parametrize("host", [False, True])
def test_pipelined_equals_plain(host):
    _, d = _frames()
    ref = _run(d, False, host=host)
    got = _run(d, True, host=host)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    assert np.array_equal(got[2][0], got[0][-1]) and np.array_equal(got[2][1], got[1][-1])


def test_pipelined_with_proposal_and_mode_switch():
    _, d = _frames()
    net = learn.load_net(learn.DEFAULT_WEIGHTS, 1, H // 4, W // 4)
    ref = _run(d, False, net=net)
    for kw in (dict(), dict(switch_off_at=4)):
        got = _run(d, True, net=net, **kw)
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), kw
    net.close()


def test_pipelined_stage_reads_wait():
    """A buffer read right after a pipelined frame sees that frame's refinement."""
    frames, d = _frames(3)
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    eng = bm.BriefMatch(prm)
    eng.setup()
    eng.set_pipelined(True)
    outs = []
    for k in range(3):
        eng.frame(d[k].data_ptr(), True)
        outs.append(eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, H, W))
    eng.clean()
    ref = bm.FlowEngine(prm)
    for k, f in enumerate(frames):
        u, v = ref.process_frame(f)
        assert np.array_equal(outs[k][0], u) and np.array_equal(outs[k][1], v), k
    ref.clean()


@pytest.mark.parametrize("pipelined", [False, True])
def test_proposal_side_stream_equals_context_stream(pipelined):
    """The network on the context's side stream (concurrent with up-sampling and
    descriptors) gives the same flows as on the context stream."""
    _, d = _frames()
    net = learn.load_net(learn.DEFAULT_WEIGHTS, 1, H // 4, W // 4)
    ref = _run(d, pipelined, net=net, side=False)
    got = _run(d, pipelined, net=net, side=True)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    net.close()
