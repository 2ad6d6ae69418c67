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
