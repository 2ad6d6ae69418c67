"""CPU checks of the oracle against independent numpy restatements on small inputs
and against the invariants the reference algorithm keeps."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from bmtest import hamming_at, random_field, random_image


def _np_features(I, pattern, N):
    # briefmatch_cuda.cu:82-124, vectorised
    sy, sx = I.shape
    ys, xs = np.mgrid[0:sy, 0:sx]
    ns = (N + 31) // 32
    F = np.zeros((sy * sx, ns), np.uint32)
    for s in range(N):
        o = np.trunc(pattern[4 * s:4 * s + 4]).astype(np.int64)
        x1 = np.clip(xs + o[0], 0, sx - 1)
        y1 = np.clip(ys + o[1], 0, sy - 1)
        x2 = np.clip(xs + o[2], 0, sx - 1)
        y2 = np.clip(ys + o[3], 0, sy - 1)
        bit = (I[y1, x1] > I[y2, x2]).ravel().astype(np.uint32)
        F[:, s // 32] |= bit << np.uint32(s % 32)
    return F


@pytest.mark.parametrize("N", [1, 31, 33, 128])
def test_features_against_numpy(N):
    rng = np.random.default_rng(N)
    I = random_image(rng, 41, 29)
    pattern = (rng.normal(0, 6, size=4 * N)).astype(np.float32)
    assert np.array_equal(oracle.features(I, pattern, N), _np_features(I, pattern, N))


def _np_jump_level(F1, F2, sx, sy, p, pd, dp, NX, NY, H):
    n = sx * sy
    NXo, NYo, Ho = NX.copy(), NY.copy(), H.copy()
    for y in range(sy):
        for x in range(sx):
            pix = x + y * sx
            cx, cy, h = int(NX[pix]), int(NY[pix]), int(H[pix])
            for d in ((-1, 1) if dp else (1,)):
                for xy in (0, 1):
                    q = pix + (pd * p * d if xy else sx * pd * p * d)
                    vx, vy = (int(NX[q]), int(NY[q])) if 0 <= q < n else (0, 0)
                    nx = min(max(vx, -x), sx - x - 1)
                    ny = min(max(vy, -y), sy - y - 1)
                    if (nx, ny) == (cx, cy):
                        continue
                    t = pix + nx + ny * sx
                    hc = int(np.unpackbits((F1[pix] ^ F2[t]).view(np.uint8)).sum())
                    if hc < h:
                        h, cx, cy = hc, nx, ny
            NXo[pix], NYo[pix], Ho[pix] = cx, cy, h
    return NXo, NYo, Ho


@pytest.mark.parametrize("p,pd,dp", [(4, -1, 1), (1, 1, 1), (8, 1, 0), (16, -1, 1)])
def test_jump_level_against_python(p, pd, dp):
    rng = np.random.default_rng(p)
    sx, sy, N = 23, 17, 64
    I1, I2 = random_image(rng, sx, sy), random_image(rng, sx, sy)
    pat = rng.normal(0, 3, size=4 * N).astype(np.float32)
    F1, F2 = oracle.features(I1, pat, N), oracle.features(I2, pat, N)
    NX, NY = random_field(rng, sx, sy, 5)
    H = hamming_at(F1, F2, sx, NX, NY)
    got = oracle.jump_level(F1, F2, sx, sy, N, p, pd, dp, NX, NY, H)
    want = _np_jump_level(F1, F2, sx, sy, p, pd, dp, NX, NY, H)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_match_invariants():
    rng = np.random.default_rng(3)
    sx, sy, N = 60, 40, 128
    I1 = random_image(rng, sx, sy)
    I2 = np.roll(I1, (2, 3), axis=(0, 1))
    pat = rng.normal(0, 4, size=4 * N).astype(np.float32)
    F1, F2 = oracle.features(I1, pat, N), oracle.features(I2, pat, N)
    nrm = oracle.normals(1, 2 * 2 * sx * sy)
    NX, NY, H0 = oracle.initialize(F1, F2, sx, sy, N, True)
    NXm, NYm, H = oracle.match(F1, F2, sx, sy, N, 2, 256, 1, 1, oracle.search_dist(sx), nrm)
    assert np.array_equal(H, hamming_at(F1, F2, sx, NXm, NYm))
    assert (H <= H0).all() and H.mean() < H0.mean()
    xs = np.tile(np.arange(sx), sy)
    ys = np.repeat(np.arange(sy), sx)
    assert ((xs + NXm >= 0) & (xs + NXm < sx) & (ys + NYm >= 0) & (ys + NYm < sy)).all()
    # interior pixels of a pure translation mostly find it
    inner = (xs > 8) & (xs < sx - 8) & (ys > 8) & (ys < sy - 8)
    hit = (NXm == 3) & (NYm == 2)
    assert hit[inner].mean() > 0.3


def test_random_search_uses_given_normals():
    rng = np.random.default_rng(4)
    sx, sy, N = 30, 20, 32
    I1, I2 = random_image(rng, sx, sy), random_image(rng, sx, sy)
    pat = rng.normal(0, 3, size=4 * N).astype(np.float32)
    F1, F2 = oracle.features(I1, pat, N), oracle.features(I2, pat, N)
    NX, NY, H = oracle.initialize(F1, F2, sx, sy, N, True)
    nrm = np.zeros(2 * sx * sy, np.float32)  # every candidate is (0,0): nothing changes
    a = oracle.random_search(F1, F2, sx, sy, N, 5.0, nrm, NX, NY, H)
    assert all(np.array_equal(x, y) for x, y in zip(a, (NX, NY, H)))
    nrm = rng.normal(size=2 * sx * sy).astype(np.float32)
    NX2, NY2, H2 = oracle.random_search(F1, F2, sx, sy, N, 5.0, nrm, NX, NY, H)
    assert (H2 <= H).all()
    changed = H2 < H
    cand_x = np.rint(5.0 * nrm[0::2])  # round half away from zero differs only at .5 ties
    assert np.array_equal(NX2[changed], np.clip(cand_x, -np.tile(np.arange(sx), sy),
                                                sx - 1 - np.tile(np.arange(sx), sy))[changed].astype(np.int16))


def test_downsample_equal_size_is_conversion():
    rng = np.random.default_rng(5)
    NX, NY = random_field(rng, 20, 10, 4)
    U, V = oracle.downsample(NX, NY, 20, 10, 20, 10, oracle.gauss_taps(0.5))
    assert np.array_equal(U.ravel(), NX.astype(np.float32)) and np.array_equal(V.ravel(), NY.astype(np.float32))


def test_downsample_constant_field():
    sx, sy, W, H = 87, 58, 30, 20
    n = sx * sy
    NX = np.full(n, 6, np.int16)
    NY = np.full(n, -3, np.int16)
    U, V = oracle.downsample(NX, NY, sx, sy, W, H, oracle.gauss_taps(0.8))
    assert np.allclose(U, 6 * np.float32(W) / sx, atol=1e-5) and np.allclose(V, -3 * np.float32(H) / sy, atol=1e-5)


def test_median_interior_matches_numpy():
    rng = np.random.default_rng(6)
    a = rng.normal(size=(15, 40)).astype(np.float32)
    for fs in (1, 3, 9, 13):
        ks = fs // 2
        h = oracle.median1d(a, 1, fs)
        want = np.array([[np.median(a[y, x - ks:x + ks + 1]) for x in range(ks, 40 - ks)] for y in range(15)])
        assert np.array_equal(h[:, ks:40 - ks], want.astype(np.float32))
        v = oracle.median1d(a, 0, fs)
        want = np.array([[np.median(a[y - ks:y + ks + 1, x]) for x in range(40)] for y in range(ks, 15 - ks)])
        assert np.array_equal(v[ks:15 - ks], want.astype(np.float32))


def test_median_guard_and_row_wrap():
    # linear index: the window of (0, y) reaches the end of row y-1; outside the plane it reads 0
    a = np.arange(1, 13, dtype=np.float32).reshape(3, 4)
    h = oracle.median1d(a, 1, 3)
    assert h[1, 0] == np.median([4, 5, 6]) and h[0, 0] == np.median([0, 1, 2])
    v = oracle.median1d(a, 0, 3)
    assert v[0, 0] == np.median([0, 1, 5]) and v[2, 3] == np.median([8, 12, 0])


def test_trilateral_constant_and_bounds():
    rng = np.random.default_rng(7)
    H, W = 20, 30
    I = random_image(rng, W, H)
    U = np.full((H, W), 2.5, np.float32)
    V = np.full((H, W), -1.0, np.float32)
    Uo, Vo = oracle.trilateral(U, V, U, V, I, 0.16, 0.01, 25.0)
    assert np.allclose(Uo, 2.5, atol=1e-5) and np.allclose(Vo, -1.0, atol=1e-5)
    U = rng.normal(size=(H, W)).astype(np.float32)
    Uo, _ = oracle.trilateral(U, V, U, V, I, 0.16, 0.01, 25.0)
    assert Uo.min() >= U.min() - 1e-5 and Uo.max() <= U.max() + 1e-5


def test_upsample_constant_and_identity():
    img = np.full((12, 17), 77.0, np.float32)
    up = oracle.upsample(img, 30, 21)
    assert np.allclose(up, 77.0, atol=1e-3)
    rng = np.random.default_rng(8)
    img = random_image(rng, 20, 15)
    assert np.allclose(oracle.upsample(img, 20, 15), img, atol=1e-3)


def test_epe():
    U = np.zeros(4, np.float32)
    V = np.zeros(4, np.float32)
    assert oracle.epe(U, V, np.array([3, 0, 0, 2e9], np.float32), np.array([4, 0, 0, 0], np.float32)) == 5.0 / 3


def test_search_dist():
    # briefmatch.cpp:271
    assert oracle.search_dist(2969) == np.float32(np.sqrt(np.ceil(np.float32(2969) * np.float32(0.5) / np.float32(3))))


def _pix_hamming(F1, F2, p, q):
    return int(sum(bin(int(a) ^ int(b)).count("1") for a, b in zip(F1[p], F2[q])))


def _setup_pair(seed, sx, sy, N):
    rng = np.random.default_rng(seed)
    pattern = np.clip(rng.normal(0, 4, 4 * N), -12, 12).astype(np.float32)
    F1 = oracle.features(random_image(rng, sx, sy), pattern, N)
    F2 = oracle.features(random_image(rng, sx, sy), pattern, N)
    return rng, F1, F2


@pytest.mark.parametrize("first", [True, False])
def test_seed_against_python(first):
    """oracle.seed (vectorised) against a per-pixel loop of the seeding rule."""
    sx, sy, N = 23, 17, 64
    rng, F1, F2 = _setup_pair(5, sx, sy, N)
    NX0, NY0 = random_field(rng, sx, sy, 5) if not first else (None, None)
    w4, h4 = 6, 5
    pred = np.zeros((h4, w4, 3), np.float32)
    pred[..., :2] = rng.uniform(-2, 2, (h4, w4, 2))
    pred[..., 2] = rng.choice([-1.0, 1.0], (h4, w4))
    scx, scy = np.float32(sx) / np.float32(w4), np.float32(sy) / np.float32(h4)
    NX, NY, H = oracle.seed(F1, F2, sx, sy, N, first, pred, w4, h4, scx, scy, 0.0, NX0, NY0)
    IX, IY, IH = oracle.initialize(F1, F2, sx, sy, N, first, NX0, NY0)
    for y in range(sy):
        for x in range(sx):
            p = y * sx + x
            bx, by, bh = int(IX[p]), int(IY[p]), int(IH[p])
            qx = min(w4 - 1, max(0, int((np.float32(x) + np.float32(0.5)) * (np.float32(1) / scx))))
            qy = min(h4 - 1, max(0, int((np.float32(y) + np.float32(0.5)) * (np.float32(1) / scy))))
            u, v, c = pred[qy, qx]
            if c >= 0:
                cx = min(max(int(np.rint(u * scx)), -x), sx - x - 1)
                cy = min(max(int(np.rint(v * scy)), -y), sy - y - 1)
                if (cx, cy) != (bx, by):
                    h = _pix_hamming(F1, F2, p, p + cx + cy * sx)
                    if h < bh:
                        bx, by, bh = cx, cy, h
            assert (NX[p], NY[p], H[p]) == (bx, by, bh), (x, y)


@pytest.mark.parametrize("r", [1, 2])
def test_local_step_against_python(r):
    """oracle.local_step (vectorised) against a per-pixel loop: the own vector moved by
    r left, right, up, down (clamped), strictly-better accept in that order."""
    sx, sy, N = 21, 15, 32
    rng, F1, F2 = _setup_pair(7, sx, sy, N)
    NX0, NY0 = random_field(rng, sx, sy, 4)
    H0 = hamming_at(F1, F2, sx, NX0, NY0)
    NX, NY, H = oracle.local_step(F1, F2, sx, sy, N, r, NX0, NY0, H0)
    for y in range(sy):
        for x in range(sx):
            p = y * sx + x
            bx, by, bh = int(NX0[p]), int(NY0[p]), int(H0[p])
            ox, oy = bx, by
            for dx, dy in ((-r, 0), (r, 0), (0, -r), (0, r)):
                cx = min(max(ox + dx, -x), sx - x - 1)
                cy = min(max(oy + dy, -y), sy - y - 1)
                h = _pix_hamming(F1, F2, p, p + cx + cy * sx)
                if h < bh:
                    bx, by, bh = cx, cy, h
            assert (NX[p], NY[p], H[p]) == (bx, by, bh), (x, y)
    assert (H <= H0).all()
