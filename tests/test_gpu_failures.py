"""Failure paths, made on the host without any GPU fault (the reference turns every
CUDA failure into a CudaException through HANDLE_ERROR, util_cuda.h:102-112):

- every device allocation of bm_create, bm_batch_create and bm_net_create in turn
  fails (the allocator's test hook): the call returns BM_ERR_NOMEM, frees what it had
  allocated, and the next creation works and computes the same flow;
- bm_set_pattern needing a wider edge-replicated margin whose allocation fails keeps
  the previous pattern and working image in effect;
- guard bands around every engine buffer on odd sizes (37x23, N = 31 and 200), checked
  after each stage, stay intact, and the results equal those without guard bands
  (the buffers start filled with the guard byte, so a read of memory no kernel wrote
  would change them).
"""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

from briefmatch_gb300 import learn, synth  # noqa: E402
from briefmatch_gb300.proposal import ProposalNet  # noqa: E402

NOMEM = "status %d: " % bm.BM_ERR_NOMEM


@pytest.fixture(autouse=True)
def _hooks_off():
    bm.debug_fail_alloc(0)
    bm.debug_guard_bands(False)
    yield
    bm.debug_fail_alloc(0)
    bm.debug_guard_bands(False)


def _pair_flow(prm, frames, pattern=None):
    eng = bm.FlowEngine(prm)
    if pattern is not None:
        eng.set_pattern(pattern)
    eng.process_frame(frames[0])
    out = eng.process_frame(frames[1])
    eng.clean()
    return out


def _allocations_of(create):
    n0 = bm.lib().bm_debug_alloc_count()
    obj = create()
    n = bm.lib().bm_debug_alloc_count() - n0
    return obj, n


def test_context_create_out_of_memory_at_every_allocation():
    W, H = 37, 23
    prm = bm.BMParams.derive(W, H, 2.9, 2.9, N=31)
    frames = synth.make_pair(5, W, H, 3.0)[:2]
    want = _pair_flow(prm, frames)
    eng, count = _allocations_of(lambda: bm.FlowEngine(prm))
    eng.clean()
    assert count >= 20
    live0 = bm.debug_live_allocs()
    for k in range(1, count + 1):
        bm.debug_fail_alloc(k)
        with pytest.raises(bm.CudaException, match=NOMEM):
            bm.FlowEngine(prm)
        assert bm.debug_live_allocs() == live0, k  # everything allocated before the failure was freed
    bm.debug_fail_alloc(0)
    got = _pair_flow(prm, frames)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_wider_pattern_allocation_failure_keeps_previous_pattern():
    W, H = 64, 40
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    frames = synth.make_pair(8, W, H, 4.0)[:2]
    q = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    q.patchArea = prm.patchArea * 3.0
    wide = q.make_pattern(77)
    eng = bm.FlowEngine(prm)
    want = (eng.process_frame(frames[0]), eng.process_frame(frames[1]))[1]
    bm.debug_fail_alloc(1)
    with pytest.raises(bm.CudaException, match=NOMEM):
        eng.set_pattern(wide)
    bm.debug_fail_alloc(0)
    eng.reset_sequence()
    eng.set_rng_position(0)
    eng.process_frame(frames[0])
    got = eng.process_frame(frames[1])
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    # the wider pattern installs once memory is there, and equals a fresh context with it
    eng.set_pattern(wide)
    eng.reset_sequence()
    eng.set_rng_position(0)
    eng.process_frame(frames[0])
    got = eng.process_frame(frames[1])
    eng.clean()
    ref = _pair_flow(prm, frames, wide)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


def test_batch_create_out_of_memory_at_every_allocation():
    sizes = [(40, 28), (52, 36)]
    params = [bm.BMParams.derive(w, h, 2.0, 2.0, N=64) for w, h in sizes]
    frames = [synth.make_pair(30 + k, w, h, 3.0)[:2] for k, (w, h) in enumerate(sizes)]
    b, count = _allocations_of(lambda: bm.Batch(params))
    b.close()
    assert count >= 4
    live0 = bm.debug_live_allocs()
    for k in range(1, count + 1):
        bm.debug_fail_alloc(k)
        with pytest.raises(bm.CudaException, match=NOMEM):
            bm.Batch(params)
        assert bm.debug_live_allocs() == live0, k
    bm.debug_fail_alloc(0)
    b = bm.Batch(params)
    b.load_frames(b.pack_frames(frames))
    b.run()
    b.synchronize()
    for (gu, gv), p, f in zip(b.read_flows(), params, frames):
        wu, wv = _pair_flow(p, f)
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv)
    b.close()


def test_net_create_out_of_memory_at_every_allocation():
    net, count = _allocations_of(lambda: ProposalNet(1, 8, 12))
    net.close()
    assert count >= 10
    live0 = bm.debug_live_allocs()
    for k in range(1, count + 1):
        bm.debug_fail_alloc(k)
        with pytest.raises(bm.CudaException, match=NOMEM):
            ProposalNet(1, 8, 12)
        assert bm.debug_live_allocs() == live0, k
    bm.debug_fail_alloc(0)
    ProposalNet(1, 8, 12).close()


def _stages(prm, frames, pattern, check):
    """Every stage of a pair through the stage entry points, `check()` after each;
    returns the field, the down-sampled and the refined flow."""
    eng = bm.BriefMatch(prm)
    eng.setup()
    eng.set_pattern(pattern)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    check()
    ups = []
    for f in frames:
        d8 = torch.from_numpy(f).cuda()
        up = torch.empty(prm.sy, prm.sx, device="cuda")
        eng.upsample_u8(d8.data_ptr(), up.data_ptr())
        ups.append(up)
        check()
    eng.features(ups[0].data_ptr(), 0)
    check()
    eng.features(ups[1].data_ptr(), 1)
    check()
    eng.initialize(True)
    check()
    pd = -1
    for _ in range(prm.iterations):
        eng.propagate(pd)
        check()
        eng.random_search()
        check()
        pd = -pd
    eng.downsample()
    check()
    prev = torch.from_numpy(frames[0].astype(np.float32)).cuda()
    eng.process(prev.data_ptr())
    check()
    rgb = eng.compute_colors()
    check()
    n = prm.sx * prm.sy
    field = eng.read_buffer(bm.BM_BUF_FLOW, np.uint32, n)
    cost = eng.read_buffer(bm.BM_BUF_COST, np.uint16, n)
    down = eng.read_buffer(bm.BM_BUF_FLOW_IN, np.float32)
    out = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32)
    check()
    eng.clean()
    return field, cost, down, out, rgb


@pytest.mark.parametrize("N,u", [(31, 2.9), (200, 1.7)])
def test_guard_bands_intact_after_every_stage(N, u):
    W, H = 37, 23
    prm = bm.BMParams.derive(W, H, u, u, N=N)
    frames = synth.make_pair(13, W, H, 3.0)[:2]
    pattern = prm.make_pattern(21)
    want = _stages(prm, frames, pattern, lambda: None)
    bm.debug_guard_bands(True)
    counts = []
    got = _stages(prm, frames, pattern, lambda: counts.append(bm.debug_check_guards()))
    bm.debug_guard_bands(False)
    assert max(counts) >= 20  # the context's buffers were guarded
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_guard_bands_intact_in_batch_and_network():
    sizes = [(37, 23), (41, 29)]
    params = [bm.BMParams.derive(w, h, 2.9, 2.9, N=128) for w, h in sizes]
    frames = [synth.make_pair(60 + k, w, h, 3.0)[:2] for k, (w, h) in enumerate(sizes)]

    def run_batch():
        b = bm.Batch(params)
        b.load_frames(b.pack_frames(frames))
        net = learn.load_net(learn.DEFAULT_WEIGHTS, 1, max(h for _, h in sizes) // 4, max(w for w, _ in sizes) // 4)
        b.set_proposal(net, 0.5, 1, 8)
        b.set_schedule(per_pair=1, use_graph=0)
        b.run()
        b.synchronize()
        flows = b.read_flows()
        n_checked = bm.debug_check_guards()
        b.close()
        net.close()
        return flows, n_checked

    want, _ = run_batch()
    bm.debug_guard_bands(True)
    got, n_checked = run_batch()
    bm.debug_guard_bands(False)
    assert n_checked >= 20
    for (gu, gv), (wu, wv) in zip(got, want):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv)
