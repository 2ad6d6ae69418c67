"""The learned proposal wired into matching: the seeded initialisation against the
oracle's restatement (bit-exact field and costs), a seeded frame sequence against
oracle.Sequence with the same proposal, training on BriefMatch's own flows, and
the gain of the committed weights (EPE against the truth at equal schedules)."""
from __future__ import annotations

import os

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle
from bmtest import engine_field, engine_normals, hamming_at, make_engine, random_field, set_field, small_params

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

from briefmatch_gb300 import learn, synth  # noqa: E402
from briefmatch_gb300.proposal import ProposalNet  # noqa: E402

FLOW_TOL = 1e-4


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _features(eng, prm, pattern, seed):
    f1, f2, _, _ = synth.make_pair(seed, prm.sx, prm.sy, 6.0)
    i1, i2 = f1.astype(np.float32), f2.astype(np.float32)
    d1, d2 = _dev(i1), _dev(i2)
    eng.features(d1.data_ptr(), 0)
    eng.features(d2.data_ptr(), 1)
    torch.cuda.synchronize()
    return oracle.features(i1, pattern, prm.N), oracle.features(i2, pattern, prm.N)


def _prediction(rng, w4, h4, vmax):
    """Random proposal: vectors in quarter-resolution pixels, logits away from 0."""
    pred = np.empty((h4, w4, 3), np.float32)
    pred[..., 0] = rng.uniform(-vmax, vmax, (h4, w4))
    pred[..., 1] = rng.uniform(-vmax, vmax, (h4, w4))
    mag = rng.uniform(0.25, 3.0, (h4, w4))
    pred[..., 2] = np.where(rng.uniform(size=(h4, w4)) < 0.7, mag, -mag)
    return pred


@pytest.mark.parametrize("first", [True, False])
def test_seed_matches_oracle(first):
    prm = small_params(104, 72, 1.5, 1.5, N=128)
    eng, pattern = make_engine(prm)
    F1, F2 = _features(eng, prm, pattern, seed=21)
    rng = np.random.default_rng(5)
    NX0 = NY0 = None
    if not first:
        NX0, NY0 = random_field(rng, prm.sx, prm.sy, 8)
        set_field(eng, NX0, NY0, np.zeros(prm.sx * prm.sy, np.uint16))
    w4, h4 = (prm.sx + 4) // 5, (prm.sy + 4) // 5        # non-integer cell scale
    pred = _prediction(rng, w4, h4, 3.0)
    d_pred = _dev(pred)
    bm.seed(eng, first, d_pred.data_ptr(), w4, h4, 0.5)
    nx, ny, cost, _ = engine_field(eng)
    scx = np.float32(prm.sx) / np.float32(w4)
    scy = np.float32(prm.sy) / np.float32(h4)
    NX, NY, H = oracle.seed(F1, F2, prm.sx, prm.sy, prm.N, first, pred, w4, h4, scx, scy, 0.0, NX0, NY0)
    assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)
    # never worse than the plain initialisation, and the proposal was used somewhere
    _, _, H0 = oracle.initialize(F1, F2, prm.sx, prm.sy, prm.N, first, NX0, NY0)
    assert (cost <= H0).all() and (cost < H0).any()


@pytest.mark.parametrize("r", [1, 3])
def test_local_step_matches_oracle(r):
    prm = small_params(96, 64, 1.5, 1.5, N=64)
    eng, pattern = make_engine(prm)
    F1, F2 = _features(eng, prm, pattern, seed=23)
    rng = np.random.default_rng(r)
    NX0, NY0 = random_field(rng, prm.sx, prm.sy, 6)
    H0 = hamming_at(F1, F2, prm.sx, NX0, NY0)
    set_field(eng, NX0, NY0, H0)
    bm.local_step(eng, r)
    nx, ny, cost, _ = engine_field(eng)
    NX, NY, H = oracle.local_step(F1, F2, prm.sx, prm.sy, prm.N, r, NX0, NY0, H0)
    assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)
    assert (cost <= H0).all() and (cost < H0).any()


def test_seed_rejects_bad_arguments():
    prm = small_params(64, 48)
    eng, _ = make_engine(prm)
    d = torch.zeros(4, 4, 3, device="cuda")
    with pytest.raises(bm.BriefMatchException):
        bm.seed(eng, True, d.data_ptr(), 4, 4, 1.0)
    with pytest.raises(bm.BriefMatchException):
        bm.seed(eng, True, d.data_ptr(), 0, 4, 0.5)
    with pytest.raises(bm.BriefMatchException, match="reduce must be 1, 2 or 4"):
        bm.set_proposal_reduce(eng, 8)
    small, _ = make_engine(small_params(40, 12))
    bm.set_proposal_reduce(small, 2)
    with pytest.raises(bm.BriefMatchException, match="frame too small"):
        bm.set_proposal_reduce(small, 4)  # 12 rows < 4 * 4
    small.clean()


def _net_with_spread_logits(h4, w4, seed=3):
    """A net whose confidence logits straddle 0 (some cells seeded, some not)."""
    net = ProposalNet(1, h4, w4)
    rng = np.random.default_rng(seed)
    p = net.params()
    p += rng.normal(0, 0.05, p.size).astype(np.float32)
    net.set_params(p)
    return net


@pytest.mark.parametrize("local,reduce", [((), 1), ((2, 1), 1), ((), 2), ((2, 1), 4)])
def test_seeded_sequence_matches_oracle(local, reduce):
    """The seeded frame loop against the oracle's, with the network on the frames
    (cells of 4 pixels) and on frames reduced 2x and 4x (cells of 8 and 16, bm_set_proposal_reduce)."""
    W, H = 88, 64
    prm = small_params(W, H, 2.0, 2.0, N=64)
    eng, pattern = make_engine(prm, pattern_seed=4)
    h4, w4 = H // reduce // 4, W // reduce // 4
    net = _net_with_spread_logits(H // 4, W // 4)
    it, jf = 1, 8
    bm.set_proposal(eng, net, 0.5, it, jf)
    if reduce != 1:
        bm.set_proposal_reduce(eng, reduce)
    if local:
        bm.set_local_steps(eng, len(local), local[0])

    def pred_fn(prev_u8, cur_u8, check=True):
        d0, d1 = _dev(prev_u8), _dev(cur_u8)
        out = torch.empty(h4, w4, 3, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        net.prepare(0, d0.data_ptr(), d1.data_ptr(), W, H, st, reduce=reduce)
        net.forward(1, h4, w4, out.data_ptr(), st)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        if check:
            assert (o[..., 2] >= 0).any() and (o[..., 2] < 0).any()
        return o

    frames, _ = synth.make_sequence(8, W, H, 4, vmax=5.0)
    # centre the confidence logits of the first pair on 0 (the head's logit bias is
    # the last parameter), so that some cells are seeded and some are not even on the
    # few cells of a 4x reduced input
    p = net.params()
    p[-1] -= float(np.median(pred_fn(frames[0], frames[1], check=False)[..., 2]))
    net.set_params(p)

    normals_cache = {}

    def normals_fn(call, n):
        if call not in normals_cache:
            normals_cache[call] = engine_normals(eng, call)
        return normals_cache[call]

    seq = oracle.Sequence(prm.as_dict(), pattern, normals_fn, nn=eng.nn_indices(),
                          proposal=(pred_fn, 0.0, it, jf, local, reduce))
    for k, f in enumerate(frames):
        d = _dev(f)
        u = torch.empty(H, W, device="cuda")
        v = torch.empty(H, W, device="cuda")
        eng.frame(d.data_ptr(), True, u.data_ptr(), v.data_ptr(), True)
        torch.cuda.synchronize()
        nx, ny, cost, _ = engine_field(eng)
        d_up = torch.empty(prm.sy, prm.sx, device="cuda")
        eng.upsample_u8(d.data_ptr(), d_up.data_ptr())
        torch.cuda.synchronize()
        o = seq.frame(f, up=d_up.cpu().numpy())
        if k == 0:
            continue
        assert np.array_equal(nx, seq.NX) and np.array_equal(ny, seq.NY) and np.array_equal(cost, seq.H)
        err = max(np.abs(u.cpu().numpy() - o[0]).max(), np.abs(v.cpu().numpy() - o[1]).max())
        assert err <= FLOW_TOL, err
    # the random stream advanced by the proposal's iteration count per pair
    assert eng.rng_position() == 3 * it


def test_detached_proposal_is_plain():
    W, H = 96, 64
    prm = small_params(W, H, 2.0, 2.0, N=64)
    f1, f2, _, _ = synth.make_pair(17, W, H, 5.0)
    outs = []
    for attach in (False, True):
        eng = bm.FlowEngine(prm)
        if attach:
            net = _net_with_spread_logits(H // 4, W // 4)
            bm.set_proposal(eng, net, 0.5, 1, 4)
            bm.set_proposal(eng, None)
        eng.process_frame(f1)
        outs.append(eng.process_frame(f2))
        eng.clean()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("reduce", [1, 2])
def test_batch_seeded_equals_single_contexts(reduce):
    """A batch with a proposal attached gives, for every pair of uneven size, what a
    fresh context with the same proposal (and input reduction) attached gives."""
    sizes = [(96, 64), (120, 72), (72, 56)]
    params = [small_params(w, h, 2.0, 2.0, N=64) for w, h in sizes]
    frames = [synth.make_pair(60 + k, w, h, 5.0)[:2] for k, (w, h) in enumerate(sizes)]
    net = _net_with_spread_logits(max(h for _, h in sizes) // 4, max(w for w, _ in sizes) // 4)
    want = []
    for p, (f0, f1) in zip(params, frames):
        eng = bm.FlowEngine(p)
        bm.set_proposal(eng, net, 0.5, 1, 8)
        bm.set_proposal_reduce(eng, reduce)
        eng.process_frame(f0)
        want.append(eng.process_frame(f1))
        eng.clean()
    b = bm.Batch(params)
    b.set_proposal(net, 0.5, 1, 8)
    b.set_proposal_reduce(reduce)
    b.set_local_steps(0, 1)
    with pytest.raises(bm.BriefMatchException):
        b.set_schedule(per_pair=0)
    for use_graph, streams in ((0, 1), (1, 1), (1, 2), (0, 3)):
        b.set_schedule(per_pair=1, use_graph=use_graph, streams=streams)
        b.load_frames(b.pack_frames(frames))
        b.run()
        b.synchronize()
        for k, ((gu, gv), (wu, wv)) in enumerate(zip(b.read_flows(), want)):
            assert np.array_equal(gu, wu) and np.array_equal(gv, wv), (use_graph, k)
    b.close()


def test_batch_local_steps_equal_single_contexts():
    sizes = [(96, 64), (72, 56)]
    params = [small_params(w, h, 2.0, 2.0, N=64) for w, h in sizes]
    frames = [synth.make_pair(70 + k, w, h, 5.0)[:2] for k, (w, h) in enumerate(sizes)]
    net = _net_with_spread_logits(max(h for _, h in sizes) // 4, max(w for w, _ in sizes) // 4)
    want = []
    for p, (f0, f1) in zip(params, frames):
        eng = bm.FlowEngine(p)
        bm.set_proposal(eng, net, 0.5, 1, 8)
        bm.set_local_steps(eng, 2, 2)
        eng.process_frame(f0)
        want.append(eng.process_frame(f1))
        eng.clean()
    b = bm.Batch(params)
    b.set_proposal(net, 0.5, 1, 8)
    b.set_local_steps(2, 2)
    b.set_schedule(per_pair=1, use_graph=1, streams=2)
    b.load_frames(b.pack_frames(frames))
    b.run()
    b.synchronize()
    for k, ((gu, gv), (wu, wv)) in enumerate(zip(b.read_flows(), want)):
        assert np.array_equal(gu, wu) and np.array_equal(gv, wv), k
    b.close()


def test_training_on_engine_flows_reduces_loss():
    """A short run of the training loop on BriefMatch's own flows for a few pairs:
    the held-in loss falls and the proposal moves toward BriefMatch's flow."""
    n = 24
    f0, f1, tgt, gt = learn.build_set(torch, n, target_iterations=2, chunk=n, workers=4)
    net = ProposalNet(8, learn.TRAIN_H // 4, learn.TRAIN_W // 4)
    probe = range(8)
    l_before = learn.batch_loss(torch, net, f0, f1, tgt, probe)
    e_before, _, _ = learn.score(torch, net, f0, f1, tgt, gt, range(4))
    learn.train_net(torch, net, f0, f1, tgt, np.arange(n), epochs=20, batch=8, lr=3e-3, log=None)
    l_after = learn.batch_loss(torch, net, f0, f1, tgt, probe)
    e_after, _, _ = learn.score(torch, net, f0, f1, tgt, gt, range(4))
    assert l_after[0] < 0.8 * l_before[0], (l_before, l_after)
    assert e_after < e_before, (e_before, e_after)


WEIGHTS = learn.DEFAULT_WEIGHTS


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="trained proposal weights not present")
def test_committed_weights_gain():
    """EPE vs the truth at equal schedules, with and without the trained proposal, on
    a held-out synthetic sequence at the training size: seeding never loses, more
    than halves the error at the shortest schedule, and one seeded iteration with
    jump maximum 64 is at least as good as the plain default (2 iterations, 256)."""
    W, H = learn.TRAIN_W, learn.TRAIN_H
    net = learn.load_net(WEIGHTS, 1, H // 4, W // 4)
    rows = learn.evaluate(net, W, H, frames=5, seed=424242, schedules=((1, 4), (1, 64), (2, 256)), reps=1,
                          torch=torch)
    by = {(r["iterations"], r["jfMax"]): r for r in rows}
    for r in rows:
        assert r["seeded_epe"] <= r["plain_epe"] * 1.02, r
    assert by[(1, 4)]["seeded_epe"] < 0.5 * by[(1, 4)]["plain_epe"], by[(1, 4)]
    assert by[(1, 64)]["seeded_epe"] <= by[(2, 256)]["plain_epe"], rows
