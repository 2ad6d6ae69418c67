"""Batched pairs of uneven size: every pair of a batch equals a fresh single-pair
context on the same frames (bit for bit), for every schedule; the autotuner and
its cache; the bounded grid barrier gives up instead of hanging."""
from __future__ import annotations

import json

import numpy as np
import pytest

import briefmatch_gb300 as bm
from briefmatch_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

SIZES = [(96, 64), (130, 70), (64, 64), (200, 124), (77, 53)]


def _batch_inputs(u=2.0, N=64):
    params = [bm.BMParams.derive(w, h, u, u, N=N) for w, h in SIZES]
    frames = [synth.make_pair(20 + k, w, h, 5.0)[:2] for k, (w, h) in enumerate(SIZES)]
    return params, frames


def _single(params, frames):
    outs = []
    for p, (f0, f1) in zip(params, frames):
        eng = bm.FlowEngine(p)
        eng.process_frame(f0)
        outs.append(eng.process_frame(f1))
        eng.clean()
    return outs


@pytest.mark.parametrize("sched", [
    dict(persistent=0, snake=0, use_graph=0),
    dict(persistent=0, snake=1, use_graph=1),
    dict(persistent=1, snake=1, use_graph=0),
    dict(persistent=1, snake=0, use_graph=1),
    dict(persistent=0, snake=1, use_graph=1, wave_bytes=1),          # one pair per wave
    dict(persistent=1, snake=1, use_graph=1, wave_bytes=3 << 20),    # small waves
    dict(per_pair=1, persistent=0, snake=1, use_graph=1),
    dict(per_pair=1, persistent=0, snake=0, use_graph=0),
    dict(per_pair=1, persistent=0, snake=1, use_graph=1, streams=2),   # concurrent branches in the graph
    dict(per_pair=1, persistent=0, snake=1, use_graph=0, streams=3),
    dict(per_pair=1, persistent=0, snake=1, use_graph=1, streams=3, wave_bytes=3 << 20),
])
def test_batch_equals_single_pairs(sched):
    params, frames = _batch_inputs()
    want = _single(params, frames)
    b = bm.Batch(params)
    b.set_schedule(**sched)
    b.load_frames(b.pack_frames(frames))
    for _ in range(2):  # a replayed step gives the same result
        b.run()
        b.synchronize()
        got = b.read_flows()
        for k, ((gu, gv), (wu, wv)) in enumerate(zip(got, want)):
            assert np.array_equal(gu, wu) and np.array_equal(gv, wv), (sched, k)
    b.close()


@pytest.mark.parametrize("per_pair", [0, 1])
def test_batch_patterns_wider_and_narrower_than_margin(per_pair):
    """The per-pair schedule takes descriptors from an edge-replicated up-sampled image
    whose margin is sized for each pair's default pattern; a wider pattern set later
    falls back to the clamped descriptors.  Both equal single contexts with the same
    patterns."""
    params, frames = _batch_inputs()
    patterns = []
    for k, p in enumerate(params):
        q = bm.BMParams.derive(p.sx_in, p.sy_in, 2.0, 2.0, N=64)
        q.patchArea = p.patchArea * (4.0 if k % 2 == 0 else 0.25)
        patterns.append(q.make_pattern(50 + k))
    want = []
    for p, pat, (f0, f1) in zip(params, patterns, frames):
        eng = bm.FlowEngine(p)
        eng.set_pattern(pat)
        eng.process_frame(f0)
        want.append(eng.process_frame(f1))
        eng.clean()
    b = bm.Batch(params)
    for k, pat in enumerate(patterns):
        b.set_pattern(k, pat)
    b.set_schedule(per_pair=per_pair, persistent=0, snake=1, use_graph=1)
    b.load_frames(b.pack_frames(frames))
    b.run()
    b.synchronize()
    for k, ((gu, gv), (wu, wv)) in enumerate(zip(b.read_flows(), want)):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv), k
    b.close()


def test_batch_n128_and_unfiltered():
    params = [bm.BMParams.derive(w, h, 1.5, 1.5, N=128, filter=0) for w, h in SIZES[:3]]
    frames = [synth.make_pair(40 + k, w, h, 4.0)[:2] for k, (w, h) in enumerate(SIZES[:3])]
    want = _single(params, frames)
    b = bm.Batch(params)
    b.set_schedule(persistent=1, use_graph=1)
    b.load_frames(b.pack_frames(frames))
    b.run()
    b.synchronize()
    for (gu, gv), (wu, wv) in zip(b.read_flows(), want):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv)
    b.close()


def test_autotune_and_cache(tmp_path):
    params, frames = _batch_inputs()
    b = bm.Batch(params)
    b.load_frames(b.pack_frames(frames))
    cache = str(tmp_path / "tune.jsonl")
    rep = b.autotune(cache, reps=2)
    assert "persistent=" in rep
    line = json.loads(open(cache).read().strip().splitlines()[-1])
    assert {"key", "persistent", "blocks_per_sm", "snake", "use_graph", "wave_bytes", "per_pair", "ms"} <= set(line)
    chosen = b.schedule()
    b.close()
    b2 = bm.Batch(params)
    rep2 = b2.autotune(cache)
    assert rep2.startswith("cached")
    assert all(b2.schedule()[k] == chosen[k] for k in ("persistent", "per_pair", "wave_bytes", "snake"))
    b2.load_frames(b2.pack_frames(frames))
    b2.run()
    b2.synchronize()
    want = _single(params, frames)
    for (gu, gv), (wu, wv) in zip(b2.read_flows(), want):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv)
    b2.close()


def test_grid_barrier_gives_up():
    st, timed_out = bm.selftest_barrier(2, 2, 100000)
    assert st == bm.BM_OK and timed_out == 0
    st, timed_out = bm.selftest_barrier(2, 3, 2000)  # nobody can pass: all blocks give up
    assert st == bm.BM_ERR_TIMEOUT and timed_out == 1
    # the context stays usable
    x = torch.ones(4, device="cuda")
    assert float(x.sum()) == 4.0


def test_persistent_timeout_in_any_wave_is_reported():
    """A grid barrier that gives up in any wave of a multi-wave persistent step is
    reported by synchronize (the barrier's error word is cleared once per step, not
    per wave); the next step with the normal limit runs clean and matches single
    contexts."""
    params, frames = _batch_inputs()
    want = _single(params, frames)
    b = bm.Batch(params)
    b.load_frames(b.pack_frames(frames))
    b.set_schedule(persistent=1, per_pair=0, snake=1, use_graph=0, wave_bytes=1, spin_limit=1)  # a wave per pair
    b.run()
    with pytest.raises(bm.CudaException, match="status %d: " % bm.BM_ERR_TIMEOUT):
        b.synchronize()
    b.set_schedule(spin_limit=0)  # the default limit
    b.run()
    b.synchronize()
    for (gu, gv), (wu, wv) in zip(b.read_flows(), want):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv)
    b.close()
