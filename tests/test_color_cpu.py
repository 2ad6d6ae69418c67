"""The oracle's colour coding (briefmatch.cpp:373-421 with util/colorcode.cpp:27-74)
against a pure-Python restatement of the same expressions, and against the
reference's literal float atan2 call (libm atan2f)."""
from __future__ import annotations

import math

import numpy as np

import oracle

f32 = np.float32


def _wheel():
    RY, YG, GC, CB, BM, MR = 15, 6, 4, 11, 13, 6
    w = []
    w += [(255, 255 * i // RY, 0) for i in range(RY)]
    w += [(255 - 255 * i // YG, 255, 0) for i in range(YG)]
    w += [(0, 255, 255 * i // GC) for i in range(GC)]
    w += [(0, 255 - 255 * i // CB, 255) for i in range(CB)]
    w += [(255 * i // BM, 0, 255) for i in range(BM)]
    w += [(255, 0, 255 - 255 * i // MR) for i in range(MR)]
    return w


def _py_colors(U, V, maxmot):
    """computeColors / computeColor with numpy float32 for every float variable and
    Python floats (doubles) for the double expressions."""
    wheel = _wheel()
    ncols = len(wheel)

    def unknown(u, v):
        return abs(u) > 1e9 or abs(v) > 1e9 or u != u or v != v

    maxrad = f32(-1)
    for u, v in zip(U.ravel(), V.ravel()):
        if not unknown(u, v):
            maxrad = max(maxrad, f32(np.sqrt(f32(u * u) + f32(v * v), dtype=f32)))
    if maxmot > 0:
        maxrad = f32(maxmot)
    if maxrad == 0:
        maxrad = f32(1)
    out = np.zeros(U.shape + (3,), np.uint8)
    flat = out.reshape(-1, 3)
    for i, (u, v) in enumerate(zip(U.ravel(), V.ravel())):
        if unknown(u, v):
            continue
        fx, fy = f32(u / maxrad), f32(v / maxrad)
        rad = f32(np.sqrt(f32(fx * fx) + f32(fy * fy), dtype=f32))
        at = f32(math.atan2(-float(fy), -float(fx)))
        a = f32(float(at) / math.pi)
        fk = f32((float(a) + 1.0) / 2.0 * (ncols - 1))
        k0 = int(fk)
        k1 = (k0 + 1) % ncols
        f = f32(fk - f32(k0))
        for b in range(3):
            col0 = f32(wheel[k0][b] / 255.0)
            col1 = f32(wheel[k1][b] / 255.0)
            col = f32(f32(f32(1) - f) * col0) + f32(f * col1)
            col = f32(col)
            if rad <= 1:
                col = f32(f32(1) - f32(rad * f32(f32(1) - col)))
            else:
                col = f32(float(col) * 0.75)
            flat[i, b] = int(255.0 * float(col))
    return out


def _field(rng, h, w, scale):
    ang = rng.uniform(-np.pi, np.pi, size=(h, w))
    mag = rng.uniform(0, 1.6, size=(h, w)) * scale
    U = (mag * np.cos(ang)).astype(f32)
    V = (mag * np.sin(ang)).astype(f32)
    U[0, :4] = [0, np.nan, 2e9, -3e9]
    V[0, :4] = [0, 0, 0, 1]
    return U, V


def test_oracle_colors_equal_python_restatement():
    rng = np.random.default_rng(5)
    U, V = _field(rng, 20, 40, 3.0)
    for maxmot in (3.0, 0.0):
        want = _py_colors(U, V, maxmot)
        got = oracle.flow_colors(U, V, maxmot)
        assert np.array_equal(got, want), maxmot
    # every wheel entry is hit, vectors inside and outside the unit disc occur
    assert np.unique(got.reshape(-1, 3), axis=0).shape[0] > 300


def test_oracle_colors_against_libm_atan2f():
    """The reference calls the host's float atan2; glibc's is not correctly rounded on
    some inputs, which moves a byte by one on rare pixels only."""
    rng = np.random.default_rng(6)
    U, V = _field(rng, 512, 512, 5.0)
    a = oracle.flow_colors(U, V, 5.0).astype(int)
    b = oracle.flow_colors(U, V, 5.0, libm_atan2f=True).astype(int)
    d = np.abs(a - b)
    assert d.max() <= 1
    assert (d > 0).mean() < 1e-3
