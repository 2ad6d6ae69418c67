"""Training-data generation of the learned proposal (briefmatch_gb300/learn.py), on
the CPU: each kind yields 512x384 pairs with quarter-resolution truth, and a
"crops" pair is a window of an independent pair of uneven size, frames and truth
cut at the same place."""
from __future__ import annotations

import numpy as np
import pytest

from briefmatch_gb300 import learn, synth


@pytest.mark.parametrize("kind", ["pairs", "crops"])
def test_group_shapes(kind):
    g = learn._group(11, kind)
    assert len(g) == learn.PAIRS_PER_GROUP[kind]
    for f0, f1, uq, vq in g:
        assert f0.shape == f1.shape == (learn.TRAIN_H, learn.TRAIN_W) and f0.dtype == np.uint8
        assert uq.shape == vq.shape == (learn.TRAIN_H // 4, learn.TRAIN_W // 4)
        assert f0.flags.c_contiguous and f1.flags.c_contiguous


def test_crops_are_windows_of_an_uneven_pair():
    g = 7
    rng = np.random.default_rng([learn.CROP_SEED, g])
    W = 4 * int(rng.integers(learn.TRAIN_W // 4, learn.CROP_MAX_W // 4 + 1))
    H = 4 * int(rng.integers(learn.TRAIN_H // 4, learn.CROP_MAX_H // 4 + 1))
    assert learn.TRAIN_W <= W <= learn.CROP_MAX_W and learn.TRAIN_H <= H <= learn.CROP_MAX_H
    f0, f1, u, v = synth.make_pair(learn.CROP_SEED + g, W, H, vmax=15.0)
    for c0, c1, uq, vq in learn._group(g, "crops"):
        x0 = int(rng.integers(0, W - learn.TRAIN_W + 1))
        y0 = int(rng.integers(0, H - learn.TRAIN_H + 1))
        win = (slice(y0, y0 + learn.TRAIN_H), slice(x0, x0 + learn.TRAIN_W))
        assert np.array_equal(c0, f0[win]) and np.array_equal(c1, f1[win])
        assert np.array_equal(uq, learn.quarter(u[win]) / 4.0) and np.array_equal(vq, learn.quarter(v[win]) / 4.0)


def test_unknown_kind_rejected():
    with pytest.raises(ValueError):
        learn._group(0, "frames")


class _FakeNet:
    """Records the snapshot/restore calls of a SpikeGuard; the 'state' is the step at
    which each slot was written."""

    def __init__(self):
        self.slots = {}
        self.calls = []
        self.now = 0

    def snapshot(self, slot, stream=0):
        self.slots[slot] = self.now
        self.calls.append(("snapshot", slot, self.now))

    def restore(self, slot, stream=0):
        assert slot in self.slots
        self.calls.append(("restore", slot, self.slots[slot]))


def _drive(guard, net, losses):
    rolled = []
    for step, flow in enumerate(losses, start=1):
        net.now = step
        if guard.step(step, flow):
            rolled.append(step)
    return rolled


def test_spike_guard_restores_the_newest_validated_snapshot():
    net = _FakeNet()
    g = learn.SpikeGuard(net, factor=8.0, window=20, every=50)
    losses = [0.02] * 120
    losses[74] = 1.0    # step 75: a spike between snapshots
    losses[100] = 1.0   # step 101: a spike right after the step-100 snapshot, before it is validated
    rolled = _drive(g, net, losses)
    assert rolled == [75, 101]
    snaps = [c for c in net.calls if c[0] == "snapshot"]
    restores = [c for c in net.calls if c[0] == "restore"]
    # the first snapshot once the window is full (step 20), then every 50 steps
    assert [c[2] for c in snaps] == [20, 50, 100]
    # step 75 goes back to the step-50 snapshot (validated at 51); step 101 cannot use
    # the unvalidated step-100 snapshot and goes back to the step-50 one again
    assert [c[2] for c in restores] == [50, 50]
    # the validated slot is never overwritten
    assert snaps[1][1] != snaps[0][1] and snaps[2][1] != snaps[1][1]
    assert g.rollbacks == 2


def test_spike_guard_without_a_snapshot_only_skips():
    net = _FakeNet()
    g = learn.SpikeGuard(net, factor=8.0, window=10, every=100)
    losses = [0.5] * 10 + [5.0] + [0.5] * 3
    rolled = _drive(g, net, losses)
    # step 10 fills the window and writes the first snapshot; step 11 spikes before it
    # is validated: nothing to restore, the step is only left out
    assert rolled == [11]
    assert not [c for c in net.calls if c[0] == "restore"]
    assert g.rollbacks == 0
    # the next steady step writes a fresh snapshot
    assert [c[2] for c in net.calls if c[0] == "snapshot"] == [10, 12]
