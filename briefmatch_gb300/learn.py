"""Training and evaluation of the learned flow proposal.

  python -m briefmatch_gb300.learn train [--pairs 30000 --epochs 50 --out PATH]
  python -m briefmatch_gb300.learn eval [--weights PATH]

Training data: seeded synthetic 512x384 pairs (briefmatch_gb300.synth) -- consecutive
pairs of sequences, independent pairs, or 512x384 windows of independent pairs of
uneven size (`--data`); targets: the flow BriefMatch itself computes for each pair
(the engine with 4 iterations, the batch API), averaged to quarter resolution.  The network is trained on the GPU by
the engine's own kernels (bm_net_train_step: forward, backward and Adam on the
tensor cores).  PyTorch only holds device buffers.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "proposal_512x384_u2.9_N128.f32")
TRAIN_W, TRAIN_H, TRAIN_U, TRAIN_N = 512, 384, 2.9, 128
TRAIN_SEED = 7_000_000


SEQ_FRAMES = 8
CROP_SEED = 9_000_000
CROPS_PER_FRAME = 2
CROP_MAX_W, CROP_MAX_H = 1920, 1080
PAIRS_PER_GROUP = {"sequences": SEQ_FRAMES - 1, "pairs": 1, "crops": CROPS_PER_FRAME}


def _group(g, kind):
    """Training group g, a list of (frame0, frame1, quarter-resolution truth u, v in
    quarter-resolution pixels):

    - "sequences": the 7 consecutive pairs of 8-frame sequence g (flow redrawn per
      pair, each frame warped from the previous one, as in the sequence workload);
    - "pairs": the single independent pair g;
    - "crops": two 512x384 windows, at random places, of one independent pair whose
      size is drawn as the batched workload draws it (width U[512,1920], height
      U[384,1080], multiples of 4).  The synthetic flow's zoom and rotation act about
      the frame's centre, so its motions grow with the frame: windows of large
      frames carry the motions that large pairs have, which 512x384 frames never
      show."""
    from briefmatch_gb300 import synth

    if kind == "sequences":
        frames, flows = synth.make_sequence(TRAIN_SEED + g, TRAIN_W, TRAIN_H, SEQ_FRAMES, vmax=15.0)
        return [(frames[k], frames[k + 1], quarter(u) / 4.0, quarter(v) / 4.0) for k, (u, v) in enumerate(flows)]
    if kind == "pairs":
        f0, f1, u, v = synth.make_pair(TRAIN_SEED + g, TRAIN_W, TRAIN_H, vmax=15.0)
        return [(f0, f1, quarter(u) / 4.0, quarter(v) / 4.0)]
    if kind != "crops":
        raise ValueError("unknown training data kind %r" % (kind,))
    rng = np.random.default_rng([CROP_SEED, g])
    W = 4 * int(rng.integers(TRAIN_W // 4, CROP_MAX_W // 4 + 1))
    H = 4 * int(rng.integers(TRAIN_H // 4, CROP_MAX_H // 4 + 1))
    f0, f1, u, v = synth.make_pair(CROP_SEED + g, W, H, vmax=15.0)
    out = []
    for _ in range(CROPS_PER_FRAME):
        x0 = int(rng.integers(0, W - TRAIN_W + 1))
        y0 = int(rng.integers(0, H - TRAIN_H + 1))
        win = (slice(y0, y0 + TRAIN_H), slice(x0, x0 + TRAIN_W))
        out.append((np.ascontiguousarray(f0[win]), np.ascontiguousarray(f1[win]), quarter(u[win]) / 4.0,
                    quarter(v[win]) / 4.0))
    return out


def quarter(a):
    """4x4 box average (drops a ragged right/bottom edge)."""
    h4, w4 = a.shape[0] // 4, a.shape[1] // 4
    return a[:h4 * 4, :w4 * 4].reshape(h4, 4, w4, 4).mean(axis=(1, 3)).astype(np.float32)


def _batch_flows(pairs, iterations):
    import briefmatch_gb300 as bm

    prm = bm.BMParams.derive(TRAIN_W, TRAIN_H, TRAIN_U, TRAIN_U, N=TRAIN_N, iterations=iterations)
    b = bm.Batch([prm] * len(pairs))
    b.set_schedule(per_pair=1, use_graph=0)
    b.load_frames(b.pack_frames(pairs))
    b.run()
    b.synchronize()
    out = [(u.copy(), v.copy()) for u, v in b.read_flows()]
    b.close()
    return out


def consistent(u, v, ub, vb, thr):
    """Forward-backward check: pixel p keeps its forward vector when the backward
    flow at p + F(p) (nearest pixel) brings it back within `thr` pixels."""
    h, w = u.shape
    ys, xs = np.mgrid[0:h, 0:w]
    qx = np.rint(xs + u).astype(np.int64)
    qy = np.rint(ys + v).astype(np.int64)
    inside = (qx >= 0) & (qx < w) & (qy >= 0) & (qy < h)
    qx, qy = np.clip(qx, 0, w - 1), np.clip(qy, 0, h - 1)
    return inside & (np.hypot(u + ub[qy, qx], v + vb[qy, qx]) < thr)


def engine_targets(pairs, iterations=4, consistency=1.0):
    """BriefMatch's own flow for each (frame0, frame1) pair, computed by the batch API
    with `iterations` propagation + random-search rounds, as [n][h4][w4][3] float32:
    u, v in quarter-resolution pixels and a validity weight.  With `consistency`
    > 0, BriefMatch also computes the backward flow of every pair; a pixel counts
    only when the two agree within `consistency` pixels, each cell's target is the
    mean over its consistent pixels and its weight their fraction."""
    fw = _batch_flows([(p[0], p[1]) for p in pairs], iterations)
    bw = _batch_flows([(p[1], p[0]) for p in pairs], iterations) if consistency > 0 else None
    out = np.ones((len(pairs), TRAIN_H // 4, TRAIN_W // 4, 3), np.float32)
    for k, (u, v) in enumerate(fw):
        if bw is None:
            out[k, ..., 0] = quarter(u) / 4.0
            out[k, ..., 1] = quarter(v) / 4.0
            continue
        m = consistent(u, v, bw[k][0], bw[k][1], consistency).astype(np.float32)
        cnt = quarter(m)
        safe = np.maximum(cnt, 1e-6)
        out[k, ..., 0] = np.where(cnt > 0, quarter(u * m) / safe, quarter(u)) / 4.0
        out[k, ..., 1] = np.where(cnt > 0, quarter(v * m) / safe, quarter(v)) / 4.0
        out[k, ..., 2] = cnt
    return out


def build_set(torch, n, target_iterations, chunk=256, workers=None, kind="sequences", consistency=1.0):
    """Generate n training pairs of `kind` (see _group) chunk by chunk (spawn-started
    CPU pool, so the pool never inherits a CUDA context) and keep frames and engine
    targets on the device.  Returns (frames0 [n][H][W] u8, frames1, targets
    [n][h4][w4][3], gt [n][h4][w4][2])."""
    import multiprocessing as mp

    from functools import partial

    workers = workers or min(16, os.cpu_count() or 1)
    f0 = torch.empty(n, TRAIN_H, TRAIN_W, dtype=torch.uint8, device="cuda")
    f1 = torch.empty_like(f0)
    tgt = torch.empty(n, TRAIN_H // 4, TRAIN_W // 4, 3, device="cuda")
    gt = np.empty((n, TRAIN_H // 4, TRAIN_W // 4, 2), np.float32)
    per = PAIRS_PER_GROUP[kind]
    groups = (n + per - 1) // per
    gchunk = max(1, chunk // per)
    s = 0
    with mp.get_context("spawn").Pool(workers) as pool:
        for g0 in range(0, groups, gchunk):
            part = [p for grp in pool.map(partial(_group, kind=kind), range(g0, min(groups, g0 + gchunk)))
                    for p in grp][:n - s]
            k = len(part)
            f0[s:s + k] = torch.from_numpy(np.stack([p[0] for p in part]))
            f1[s:s + k] = torch.from_numpy(np.stack([p[1] for p in part]))
            tgt[s:s + k] = torch.from_numpy(engine_targets(part, target_iterations, consistency))
            gt[s:s + k, ..., 0] = np.stack([p[2] for p in part])
            gt[s:s + k, ..., 1] = np.stack([p[3] for p in part])
            s += k
    return f0, f1, tgt, gt


SPIKE_FACTOR = 8.0     # a flow loss this many times the recent median is a spike
SPIKE_WINDOW = 200     # steps in that median
SNAPSHOT_EVERY = 500   # steps between snapshots of the training state


class SpikeGuard:
    """Loss-spike rollback of a training loop over a ProposalNet (bm_net_snapshot /
    bm_net_restore; host bookkeeping only).  Every `every` steps the training state
    goes into the snapshot slot that does not hold the newest validated snapshot; a
    snapshot counts as validated once the next step's loss, computed with it, is
    steady.  A step whose flow loss exceeds `factor` times the median of the last
    `window` steady steps restores the newest validated snapshot."""

    def __init__(self, net, stream=0, factor=SPIKE_FACTOR, window=SPIKE_WINDOW, every=SNAPSHOT_EVERY):
        from collections import deque

        self.net, self.stream, self.factor, self.every = net, stream, factor, every
        self.recent = deque(maxlen=window)
        self.good = None      # slot of the newest validated snapshot
        self.pending = None   # slot written after the previous step, validated by this one
        self.rollbacks = 0

    def step(self, step, flow):
        """Account for the loss of training step `step` (1-based); True when the step
        was a spike and the network went back to a validated snapshot (or, before the
        first one, when the step is only left out of the median)."""
        full = len(self.recent) == self.recent.maxlen
        if full and flow > self.factor * float(np.median(self.recent)):
            self.pending = None
            if self.good is not None:
                self.net.restore(self.good, self.stream)
                self.rollbacks += 1
            return True
        self.recent.append(flow)
        if self.pending is not None:
            self.good, self.pending = self.pending, None
        if len(self.recent) == self.recent.maxlen and (self.good is None or step % self.every == 0):
            self.pending = 0 if self.good is None else self.good ^ 1
            self.net.snapshot(self.pending, self.stream)
        return False


def train_net(torch, net, f0, f1, tgt, idx_train, epochs, batch, lr, seed=1, log=print, rollback=True):
    """Adam with cosine decay over `epochs` passes of idx_train; every step runs the
    engine's kernels (input preparation, forward, backward, Adam).  With `rollback` a
    SpikeGuard returns the network to a validated snapshot after a loss spike and
    training goes on with the next batches: an unclipped update can otherwise leave
    the network dead for the rest of the run.  Returns the loss history [(step, flow
    loss, confidence loss)]; a rollback appears as an entry with the flow loss
    negated."""
    h4, w4 = TRAIN_H // 4, TRAIN_W // 4
    stream = torch.cuda.current_stream().cuda_stream
    d_bt = torch.empty(batch, h4, w4, 3, device="cuda")
    rng = np.random.default_rng(seed)
    steps_per_epoch = len(idx_train) // batch
    total = max(1, steps_per_epoch * epochs)
    step = 0
    hist = []
    guard = SpikeGuard(net, stream) if rollback else None
    for ep in range(epochs):
        order = rng.permutation(idx_train)
        for k in range(steps_per_epoch):
            idx = order[k * batch:(k + 1) * batch]
            for j, i in enumerate(idx):
                net.prepare(j, f0[i].data_ptr(), f1[i].data_ptr(), TRAIN_W, TRAIN_H, stream)
            d_bt.copy_(tgt[torch.from_numpy(idx).cuda()])
            cur = lr * 0.5 * (1 + np.cos(np.pi * step / total))
            loss = net.train_step(batch, h4, w4, d_bt.data_ptr(), float(cur), 0, stream)
            step += 1
            if guard is not None and guard.step(step, float(loss[0])):
                hist.append((step, -float(loss[0]), float(loss[1])))
                if log:
                    log("step %d/%d  flow loss %.4f: spike, back to the last validated snapshot" % (step, total, loss[0]))
                continue
            if step % 50 == 0 or step == total or step == 1:
                hist.append((step, float(loss[0]), float(loss[1])))
                if log:
                    log("step %d/%d  flow loss %.4f  conf loss %.4f" % (step, total, loss[0], loss[1]))
    return hist


def batch_loss(torch, net, f0, f1, tgt, idx):
    """(flow loss, confidence loss) of the network on pairs idx, without an update."""
    h4, w4 = TRAIN_H // 4, TRAIN_W // 4
    stream = torch.cuda.current_stream().cuda_stream
    for j, i in enumerate(idx):
        net.prepare(j, f0[i].data_ptr(), f1[i].data_ptr(), TRAIN_W, TRAIN_H, stream)
    d = tgt[torch.as_tensor(list(idx), device="cuda")].contiguous()
    loss = net.train_step(len(idx), h4, w4, d.data_ptr(), 0.0, 0, stream)
    return float(loss[0]), float(loss[1])


def score(torch, net, f0, f1, tgt, gt, idx):
    """Mean end-point error (input pixels) of the proposal against BriefMatch's flow
    and against the truth, and the fraction of confident cells, over pairs idx."""
    h4, w4 = TRAIN_H // 4, TRAIN_W // 4
    stream = torch.cuda.current_stream().cuda_stream
    out = torch.empty(1, h4, w4, 3, device="cuda")
    e_tgt, e_gt, conf = [], [], []
    for i in idx:
        net.prepare(0, f0[i].data_ptr(), f1[i].data_ptr(), TRAIN_W, TRAIN_H, stream)
        net.forward(1, h4, w4, out.data_ptr(), stream)
        o = out[0].cpu().numpy()
        t = tgt[i].cpu().numpy()
        e_tgt.append(4 * np.mean(np.hypot(o[..., 0] - t[..., 0], o[..., 1] - t[..., 1])))
        e_gt.append(4 * np.mean(np.hypot(o[..., 0] - gt[i, ..., 0], o[..., 1] - gt[i, ..., 1])))
        conf.append(np.mean(o[..., 2] > 0))
    return float(np.mean(e_tgt)), float(np.mean(e_gt)), float(np.mean(conf))


DATA_KINDS = {
    "sequences": "consecutive pairs of 8-frame sequences",
    "pairs": "single pairs",
    "crops": "512x384 windows of independent pairs of uneven size (width U[512,1920], height U[384,1080])",
    "mixed": "half consecutive pairs of 8-frame sequences, half 512x384 windows of independent pairs of uneven "
             "size (width U[512,1920], height U[384,1080])",
}


def train(args):
    import torch

    from briefmatch_gb300.proposal import ProposalNet

    t0 = time.time()
    kind = "pairs" if args.single_pairs else args.data
    if kind == "mixed":
        # half sequence pairs, half windows of uneven-size independent pairs, shuffled
        # once so that the held-out pairs cover both
        half = args.pairs // 2
        a = build_set(torch, half, args.target_iterations, kind="sequences", consistency=args.consistency)
        b = build_set(torch, args.pairs - half, args.target_iterations, kind="crops", consistency=args.consistency)
        perm = np.random.default_rng(args.seed).permutation(args.pairs)
        tp = torch.from_numpy(perm).cuda()
        f0, f1, tgt = (torch.cat([x, y])[tp].contiguous() for x, y in zip(a[:3], b[:3]))
        gt = np.concatenate([a[3], b[3]])[perm]
        del a, b
    else:
        f0, f1, tgt, gt = build_set(torch, args.pairs, args.target_iterations, kind=kind,
                                    consistency=args.consistency)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    n = args.pairs
    nval = max(1, n // 20)
    net = ProposalNet(args.batch, TRAIN_H // 4, TRAIN_W // 4)
    t1 = time.time()
    hist = train_net(torch, net, f0, f1, tgt, np.arange(nval, n), args.epochs, args.batch, args.lr, args.seed,
                     log=lambda m: print(m, flush=True))
    torch.cuda.synchronize()
    t_train = time.time() - t1
    e_tgt, e_gt, conf = score(torch, net, f0, f1, tgt, gt, range(nval))
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    net.save(args.out)
    report = {"pairs": n, "heldout": nval, "size": [TRAIN_W, TRAIN_H], "epochs": args.epochs, "batch": args.batch,
              "lr": args.lr, "target_iterations": args.target_iterations, "consistency_px": args.consistency,
              "data": DATA_KINDS[kind],
              "seconds": {"data_and_targets": t_data, "train": t_train},
              "heldout_epe_vs_briefmatch_px": e_tgt, "heldout_epe_vs_truth_px": e_gt,
              "heldout_confident_fraction": conf, "loss_history": hist}
    with open(args.out + ".json", "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps({k: v for k, v in report.items() if k != "loss_history"}))


def run_sequence(torch, prm, frames_dev, net=None, conf=0.5, iterations=1, jf_max=16, reps=3, stream=None):
    """Flows of a frame sequence through one context (bm_frame, device frames), plain
    or seeded by `net`; returns (flows [pairs][2][H][W] numpy, best device ms per
    pair over `reps` timed repetitions after one warm-up)."""
    import briefmatch_gb300 as bm

    stream = stream or torch.cuda.Stream()
    H, W = prm.sy_in, prm.sx_in
    npairs = len(frames_dev) - 1
    eng = bm.BriefMatch(prm)
    eng.setup()
    eng.set_stream(stream.cuda_stream)
    if net is not None:
        bm.set_proposal(eng, net, conf, iterations, jf_max)
    u = torch.empty(npairs, H, W, device="cuda")
    v = torch.empty(npairs, H, W, device="cuda")
    best = None
    for rep in range(reps + 1):
        eng.reset_sequence()
        eng.set_rng_position(0)
        eng.frame(frames_dev[0].data_ptr(), True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(1, npairs + 1):
            eng.frame(frames_dev[k].data_ptr(), True, u[k - 1].data_ptr(), v[k - 1].data_ptr(), True)
        e1.record(stream)
        stream.synchronize()
        if rep:
            ms = e0.elapsed_time(e1) / npairs
            best = ms if best is None else min(best, ms)
    flows = np.stack([u.cpu().numpy(), v.cpu().numpy()], axis=1)
    eng.clean()
    return flows, best


def evaluate(net, W=1024, H=436, frames=8, seed=20261203, ux=2.9, N=128, vmax=15.0,
             schedules=((1, 4), (1, 16), (1, 64), (2, 256)), conf=0.5, reps=3, torch=None):
    """End-point error against the truth and device time per pair, plain and
    seeded, at each (iterations, jfMax) schedule, on a seeded synthetic sequence
    (flow redrawn per pair, |v| <= vmax)."""
    import briefmatch_gb300 as bm
    from briefmatch_gb300 import synth

    if torch is None:
        import torch
    seq, flows = synth.make_sequence(seed, W, H, frames, vmax=vmax)
    d = [torch.from_numpy(f).cuda() for f in seq]
    gt = np.stack([np.stack(f) for f in flows])
    rows = []
    for it, jf in schedules:
        prm = bm.BMParams.derive(W, H, ux, ux, N=N, iterations=it, jfMax=jf)
        fp, tp = run_sequence(torch, prm, d, None, reps=reps)
        fs, ts = run_sequence(torch, bm.BMParams.derive(W, H, ux, ux, N=N), d, net, conf, it, jf, reps=reps)
        epe = lambda f: float(np.mean(np.hypot(f[:, 0] - gt[:, 0], f[:, 1] - gt[:, 1])))
        rows.append({"iterations": it, "jfMax": jf, "plain_epe": epe(fp), "seeded_epe": epe(fs), "plain_ms": tp,
                     "seeded_ms": ts, "plain_mpx_s": W * H / (tp * 1e-3) / 1e6,
                     "seeded_mpx_s": W * H / (ts * 1e-3) / 1e6})
    return rows


def load_net(weights, max_batch=1, max_h4=512, max_w4=512):
    from briefmatch_gb300.proposal import ProposalNet

    net = ProposalNet(max_batch, max_h4, max_w4)
    net.load(weights)
    return net


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=30000)
    t.add_argument("--epochs", type=int, default=50)
    t.add_argument("--batch", type=int, default=32)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--seed", type=int, default=1)
    t.add_argument("--target-iterations", type=int, default=4)
    t.add_argument("--consistency", type=float, default=1.0,
                   help="forward-backward agreement (px) a target pixel needs; 0 keeps every pixel")
    t.add_argument("--data", default="sequences", choices=sorted(DATA_KINDS), help="training pairs")
    t.add_argument("--single-pairs", action="store_true", help="independent pairs instead of sequences (--data pairs)")
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=DEFAULT_WEIGHTS)
    e.add_argument("--width", type=int, default=1024)
    e.add_argument("--height", type=int, default=436)
    e.add_argument("--frames", type=int, default=8)
    e.add_argument("--seed", type=int, default=20261203)
    e.add_argument("--schedules", default="1/4,1/16,1/64,2/256", help="iterations/jfMax list")
    args = ap.parse_args(argv)
    if args.cmd == "train":
        train(args)
    else:
        net = load_net(args.weights, 1, args.height // 4, args.width // 4)
        sch = [tuple(int(x) for x in t.split("/")) for t in args.schedules.split(",")]
        for row in evaluate(net, args.width, args.height, args.frames, seed=args.seed, schedules=sch):
            print(json.dumps(row))


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    main()
