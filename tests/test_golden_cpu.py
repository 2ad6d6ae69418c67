"""The oracle against golden vectors recorded from the reference's own kernels
(tests/golden/make_golden.py runs kernels/briefmatch_cuda.cu and util_cuda.cu,
compiled unmodified, on a GPU): descriptors, zero initialisation, three random
searches, the down-sampling chain and the median bit-exact; Lanczos up-sampling
within 2e-3 (libm sin and IEEE division here, fast-math intrinsics in the
reference build); the cross-trilateral filter within 1e-4 px."""
from __future__ import annotations

import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("golden vectors %s not generated" % name)
    return np.load(path)


def test_upsample_golden():
    g = _load("upsample.npz")
    for k in range(3):
        out = g["out%d" % k]
        mine = oracle.upsample(g["in%d" % k], out.shape[1], out.shape[0])
        assert np.abs(mine - out).max() <= 2e-3


@pytest.mark.parametrize("N", [32, 100, 512])
def test_features_golden(N):
    g = _load("features.npz")
    F = oracle.features(g["img_N%d" % N], g["pattern_N%d" % N], N)
    assert np.array_equal(F, g["F_N%d" % N])


def test_initialize_and_random_search_golden():
    g = _load("match.npz")
    F1, F2 = g["F1"], g["F2"]
    n = F1.shape[0]
    N = 32 * F1.shape[1]
    H = 52
    W = n // H
    nx, ny, h = oracle.initialize(F1, F2, W, H, N, True)
    assert np.array_equal(nx, g["NX_init"]) and np.array_equal(ny, g["NY_init"])
    assert np.array_equal(h, np.rint(g["D_init"] * N).astype(np.uint16))
    for call in range(3):
        nx, ny, h = oracle.random_search(F1, F2, W, H, N, float(g["dist"]), g["normals%d" % call], nx, ny, h)
        assert np.array_equal(nx, g["NX_rs%d" % call]) and np.array_equal(ny, g["NY_rs%d" % call]), call
        assert np.array_equal(h, np.rint(g["D_rs%d" % call] * N).astype(np.uint16)), call


def test_downsample_golden():
    g = _load("downsample.npz")
    sx, sy, W, H = (int(v) for v in g["dims"])
    U, V = oracle.downsample(g["NX"], g["NY"], sx, sy, W, H, g["taps"], (g["nnx"], g["nny"]))
    assert np.array_equal(U, g["U"]) and np.array_equal(V, g["V"])


@pytest.mark.parametrize("fsize", [9, 13])
def test_median_and_trilateral_golden(fsize):
    g = _load("refine.npz")
    k = "_f%d" % fsize
    U, V, I = g["U" + k], g["V" + k], g["I" + k]
    Um = oracle.median1d(oracle.median1d(U, 1, fsize), 0, fsize)
    Vm = oracle.median1d(oracle.median1d(V, 1, fsize), 0, fsize)
    assert np.array_equal(Um, g["Um" + k]) and np.array_equal(Vm, g["Vm" + k])
    sE, sI, sS = (float(x) for x in g["sigmas" + k])
    Uo, Vo = oracle.trilateral(U, V, Um, Vm, I, sE * sE, sI * sI, sS * sS)
    err = max(np.abs(Uo - g["Uo" + k]).max(), np.abs(Vo - g["Vo" + k]).max())
    assert err <= 1e-4, err
