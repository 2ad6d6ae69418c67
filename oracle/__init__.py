"""The oracle: CPU restatement of the BriefMatch flow path (TEST INFRASTRUCTURE).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may use
this package, and only as the reference the engine is compared with or as the
timed CPU baseline, never as the engine.  It wraps oracle/_build/libbmoracle.so (bm_oracle.c) with numpy arrays in
the reference's layouts: float images, uint32 descriptors [sx*sy][ceil(N/32)],
int16 NX/NY, uint16 Hamming costs.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(_HERE, "_build", "libbmoracle.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise ImportError("oracle library missing at %s; run __graft_entry__.build()" % ORACLE_LIB)
        L = ctypes.CDLL(ORACLE_LIB)
        vp, i, f, u64, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint64, ctypes.c_size_t
        sig = {
            "bmo_num_threads": (i, []),
            "bmo_set_threads": (None, [i]),
            "bmo_upsample": (None, [vp, i, i, vp, i, i]),
            "bmo_u8_to_float": (None, [vp, sz, vp]),
            "bmo_features": (None, [vp, i, i, vp, i, vp]),
            "bmo_initialize": (None, [vp, vp, i, i, i, i, vp, vp, vp]),
            "bmo_jump_level": (None, [vp, vp, i, i, i, i, i, i, vp, vp, vp, vp, vp]),
            "bmo_propagate": (None, [vp, vp, i, i, i, i, i, i, vp, vp, vp]),
            "bmo_random_search": (None, [vp, vp, i, i, i, f, vp, vp, vp, vp]),
            "bmo_match": (None, [vp, vp, i, i, i, i, i, i, i, f, vp, vp, vp, vp]),
            "bmo_search_dist": (f, [i]),
            "bmo_gauss_taps": (i, [f, vp, i]),
            "bmo_downsample": (None, [vp, vp, i, i, i, i, vp, i, vp, vp, vp, vp]),
            "bmo_median1d": (None, [vp, vp, i, i, i, i]),
            "bmo_trilateral": (None, [vp, vp, vp, vp, vp, f, f, f, i, i, vp, vp]),
            "bmo_refine": (None, [vp, vp, vp, i, i, i, f, f, f, vp, vp, vp, vp]),
            "bmo_epe": (ctypes.c_double, [vp, vp, vp, vp, sz]),
            "bmo_normals": (None, [u64, sz, vp]),
            "bmo_make_pattern": (i, [i, f, u64, vp]),
            "bmo_flow_colors": (None, [vp, vp, sz, f, i, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _c(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


def _p(a):
    return a.ctypes.data


def num_threads():
    return lib().bmo_num_threads()


def set_threads(n):
    lib().bmo_set_threads(int(n))


def upsample(img, sxo, syo):
    img = _c(img, np.float32)
    syi, sxi = img.shape
    out = np.empty((syo, sxo), np.float32)
    lib().bmo_upsample(_p(img), sxi, syi, _p(out), sxo, syo)
    return out


def features(I, pattern, N):
    I = _c(I, np.float32)
    pattern = _c(pattern, np.float32)
    sy, sx = I.shape
    ns = (N + 31) // 32
    F = np.empty((sy * sx, ns), np.uint32)
    lib().bmo_features(_p(I), sx, sy, _p(pattern), N, _p(F))
    return F


def initialize(F1, F2, sx, sy, N, first, NX=None, NY=None):
    n = sx * sy
    NX = np.zeros(n, np.int16) if NX is None else _c(NX, np.int16).copy()
    NY = np.zeros(n, np.int16) if NY is None else _c(NY, np.int16).copy()
    H = np.zeros(n, np.uint16)
    lib().bmo_initialize(_p(_c(F1, np.uint32)), _p(_c(F2, np.uint32)), sx, sy, N, int(bool(first)), _p(NX), _p(NY), _p(H))
    return NX, NY, H


def _hamming_rows(A, B):
    x = np.ascontiguousarray(A ^ B)
    return np.unpackbits(x.view(np.uint8), axis=1).sum(axis=1).astype(np.int64)


def seed(F1, F2, sx, sy, N, first, pred, w4, h4, scale_x, scale_y, logit_min, NX=None, NY=None):
    """Initialisation seeded by a quarter-resolution proposal [h4][w4][3] (u, v in
    quarter-resolution pixels, confidence logit).  No reference counterpart: the
    plain initialisation (briefmatch_cuda.cu:115-139 via bmo_initialize) runs first,
    then each pixel whose cell has logit >= logit_min tries the proposal vector
    (scaled by scale_x/y, rounded half-to-even, clamped into the image) and keeps it
    only when its Hamming cost is strictly lower.  The cell of up-sampled pixel x is
    floor((x + 0.5) * (1 / scale_x)) in float32, clamped to the grid."""
    NX, NY, H = initialize(F1, F2, sx, sy, N, first, NX, NY)
    F1 = _c(F1, np.uint32)
    F2 = _c(F2, np.uint32)
    f32 = np.float32
    ys, xs = np.mgrid[0:sy, 0:sx]
    xs, ys = xs.ravel(), ys.ravel()
    inv_x, inv_y = f32(1.0) / f32(scale_x), f32(1.0) / f32(scale_y)
    qx = np.clip(((xs.astype(f32) + f32(0.5)) * inv_x).astype(np.int64), 0, w4 - 1)
    qy = np.clip(((ys.astype(f32) + f32(0.5)) * inv_y).astype(np.int64), 0, h4 - 1)
    pr = np.asarray(pred, f32).reshape(h4, w4, 3)[qy, qx]
    cand = pr[:, 2] >= f32(logit_min)
    sxv = np.clip(np.rint(pr[:, 0] * f32(scale_x)).astype(np.int64), -xs, sx - xs - 1)
    syv = np.clip(np.rint(pr[:, 1] * f32(scale_y)).astype(np.int64), -ys, sy - ys - 1)
    cand &= (sxv != NX) | (syv != NY)
    idx = np.nonzero(cand)[0]
    q = idx + sxv[idx] + syv[idx] * sx
    hs = _hamming_rows(F1[idx], F2[q])
    win = hs < H[idx].astype(np.int64)
    w = idx[win]
    NX[w] = sxv[w]
    NY[w] = syv[w]
    H[w] = hs[win]
    return NX, NY, H


def local_step(F1, F2, sx, sy, N, r, NX, NY, H):
    """Local refinement step of the seeded schedule (no reference counterpart): each
    pixel's own vector moved by r left, right, up and down (clamped into the image),
    in that order, each kept only if strictly cheaper than the best so far; all
    pixels read the same snapshot."""
    F1 = _c(F1, np.uint32)
    F2 = _c(F2, np.uint32)
    NX = _c(NX, np.int16).astype(np.int64)
    NY = _c(NY, np.int16).astype(np.int64)
    best_x, best_y, best_h = NX.copy(), NY.copy(), _c(H, np.uint16).astype(np.int64)
    ys, xs = np.mgrid[0:sy, 0:sx]
    xs, ys = xs.ravel(), ys.ravel()
    pix = np.arange(sx * sy)
    for dx, dy in ((-r, 0), (r, 0), (0, -r), (0, r)):
        tx = np.clip(NX + dx, -xs, sx - xs - 1)
        ty = np.clip(NY + dy, -ys, sy - ys - 1)
        h = _hamming_rows(F1, F2[pix + tx + ty * sx])
        win = h < best_h
        best_x = np.where(win, tx, best_x)
        best_y = np.where(win, ty, best_y)
        best_h = np.where(win, h, best_h)
    return best_x.astype(np.int16), best_y.astype(np.int16), best_h.astype(np.uint16)


def jump_level(F1, F2, sx, sy, N, p, pd, double_prop, NX, NY, H):
    NXs = _c(NX, np.int16).copy()
    NYs = _c(NY, np.int16).copy()
    NXo, NYo, Ho = NXs.copy(), NYs.copy(), _c(H, np.uint16).copy()
    lib().bmo_jump_level(_p(_c(F1, np.uint32)), _p(_c(F2, np.uint32)), sx, sy, N, p, pd, int(bool(double_prop)),
                         _p(NXs), _p(NYs), _p(NXo), _p(NYo), _p(Ho))
    return NXo, NYo, Ho


def propagate(F1, F2, sx, sy, N, pd, jf_max, double_prop, NX, NY, H):
    NX, NY, H = _c(NX, np.int16).copy(), _c(NY, np.int16).copy(), _c(H, np.uint16).copy()
    lib().bmo_propagate(_p(_c(F1, np.uint32)), _p(_c(F2, np.uint32)), sx, sy, N, pd, jf_max, int(bool(double_prop)),
                        _p(NX), _p(NY), _p(H))
    return NX, NY, H


def random_search(F1, F2, sx, sy, N, dist, normals, NX, NY, H):
    NX, NY, H = _c(NX, np.int16).copy(), _c(NY, np.int16).copy(), _c(H, np.uint16).copy()
    nrm = _c(normals, np.float32)
    lib().bmo_random_search(_p(_c(F1, np.uint32)), _p(_c(F2, np.uint32)), sx, sy, N, dist, _p(nrm), _p(NX), _p(NY), _p(H))
    return NX, NY, H


def match(F1, F2, sx, sy, N, iterations, jf_max, double_prop, first, dist, normals, NX=None, NY=None):
    n = sx * sy
    NX = np.zeros(n, np.int16) if NX is None else _c(NX, np.int16).copy()
    NY = np.zeros(n, np.int16) if NY is None else _c(NY, np.int16).copy()
    H = np.zeros(n, np.uint16)
    nrm = _c(normals, np.float32)
    assert nrm.size >= iterations * n * 2
    lib().bmo_match(_p(_c(F1, np.uint32)), _p(_c(F2, np.uint32)), sx, sy, N, iterations, jf_max, int(bool(double_prop)),
                    int(bool(first)), dist, _p(nrm), _p(NX), _p(NY), _p(H))
    return NX, NY, H


# BMParams::BMParams (briefmatch.h:67-84), with the engine's two additions (rng, seed)
PARAM_DEFAULTS = dict(sx=64, sy=64, sx_in=64, sy_in=64, N=128, iterations=2, jfMax=256, P=11, fsize=13,
                      patchArea=75.0, sigma=0.5, sEPE=0.4, sI=0.1, sS=6.0, maxmot=5.0, doubleProp=1, filter=1,
                      tInit=1, rng=0, seed=0)


def derive_params(width, height, ux=0.0, uy=0.0, patch_radius=3.0, sigma_downsampling=0.025, median_size=1.0,
                  range_spatial=0.85, **overrides):
    """OFPipeline::setParams (of_pipeline.cpp:178-190) on the BMParams defaults, in the
    reference's types: the up-sampled size is float * unsigned truncated to unsigned,
    the diagonals are sqrt of unsigned (32-bit) sums in double, each percentage is a
    float product 0.01f * value before it meets the double diagonal."""
    f32 = np.float32
    p = dict(PARAM_DEFAULTS)
    p.update(overrides)
    ux, uy = f32(ux), f32(uy)
    if ux < f32(0.1):
        ux = f32(2.740)
    if uy < f32(0.1):
        uy = f32(3.052)
    sx, sy = int(ux * f32(width)), int(uy * f32(height))
    diag_up = float(np.sqrt(float((sx * sx + sy * sy) & 0xFFFFFFFF)))
    diag_in = float(np.sqrt(float((width * width + height * height) & 0xFFFFFFFF)))
    p.update(sx=sx, sy=sy, sx_in=int(width), sy_in=int(height))
    p["patchArea"] = float(f32(float(f32(0.01) * f32(patch_radius)) * diag_up))
    p["sigma"] = float(f32(float(f32(0.01) * f32(sigma_downsampling)) * diag_up))
    p["fsize"] = int(2 * np.round(float(f32(0.005) * f32(median_size)) * diag_in) + 1)
    p["sS"] = float(f32(float(f32(0.01) * f32(range_spatial)) * diag_in))
    return p


def make_pattern(params: dict, seed=0):
    """The BRIEF sampling pattern for these parameters (briefmatch.cpp:124-148), 4N
    floats, drawn from an explicit seed (bm_oracle_params.cpp)."""
    out = np.zeros(4 * int(params["N"]), np.float32)
    if lib().bmo_make_pattern(int(params["N"]), float(params["patchArea"]), int(seed), _p(out)) != 0:
        raise ValueError("feature length out of range")
    return out


def search_dist(sx):
    return lib().bmo_search_dist(sx)


def gauss_taps(sigma):
    out = np.zeros(100, np.float32)
    P = lib().bmo_gauss_taps(sigma, _p(out), 100)
    if P < 0:
        raise ValueError("sigma too large")
    return out[:P].copy()


def downsample(NX, NY, sx, sy, sx_in, sy_in, taps, nn=None):
    """nn = (xs, ys): the device's resizeNN index tables (bm_nn_indices); None
    computes them with IEEE division."""
    taps = _c(taps, np.float32)
    U = np.zeros((sy_in, sx_in), np.float32)
    V = np.zeros((sy_in, sx_in), np.float32)
    if nn is None:
        px = py = None
    else:
        xs, ys = _c(nn[0], np.uint32), _c(nn[1], np.uint32)
        assert xs.size == sx_in and ys.size == sy_in
        px, py = _p(xs), _p(ys)
    lib().bmo_downsample(_p(_c(NX, np.int16)), _p(_c(NY, np.int16)), sx, sy, sx_in, sy_in, _p(taps), taps.size,
                         px, py, _p(U), _p(V))
    return U, V


def median1d(a, direction, fsize):
    a = _c(a, np.float32)
    sy, sx = a.shape
    out = np.empty_like(a)
    lib().bmo_median1d(_p(a), _p(out), direction, fsize, sx, sy)
    return out


def trilateral(U, V, Um, Vm, I, sEPE2, sI2, sS2):
    U, V, Um, Vm, I = (_c(a, np.float32) for a in (U, V, Um, Vm, I))
    sy, sx = U.shape
    Uo = np.empty_like(U)
    Vo = np.empty_like(V)
    lib().bmo_trilateral(_p(U), _p(V), _p(Um), _p(Vm), _p(I), sEPE2, sI2, sS2, sx, sy, _p(Uo), _p(Vo))
    return Uo, Vo


def refine(U, V, Iprev, fsize, sEPE, sI, sS):
    U, V, Iprev = (_c(a, np.float32) for a in (U, V, Iprev))
    sy, sx = U.shape
    Um, Vm, Uo, Vo = (np.empty_like(U) for _ in range(4))
    lib().bmo_refine(_p(U), _p(V), _p(Iprev), sx, sy, fsize, sEPE, sI, sS, _p(Um), _p(Vm), _p(Uo), _p(Vo))
    return Um, Vm, Uo, Vo


def epe(U, V, Ugt, Vgt):
    U, V, Ugt, Vgt = (_c(a, np.float32) for a in (U, V, Ugt, Vgt))
    return lib().bmo_epe(_p(U), _p(V), _p(Ugt), _p(Vgt), U.size)


def flow_colors(U, V, maxmot, libm_atan2f=False):
    """Colour coding of a flow field (briefmatch.cpp:373-421, colorcode.cpp:27-74):
    [h][w][3] uint8, R G B."""
    U = _c(U, np.float32)
    V = _c(V, np.float32)
    assert U.shape == V.shape
    out = np.zeros(U.shape + (3,), np.uint8)
    lib().bmo_flow_colors(_p(U), _p(V), U.size, float(maxmot), int(bool(libm_atan2f)), _p(out))
    return out


def normals(seed, count):
    out = np.empty(count, np.float32)
    lib().bmo_normals(seed, count, _p(out))
    return out


class Sequence:
    """OFPipeline-style frame loop on the CPU (of_pipeline.cpp:241-333), in the
    same order as the engine's bm_frame: the first frame primes, later frames
    produce the flow from the previous frame.

    ``up_images`` lets a caller supply the up-sampled frames (e.g. the engine's,
    to take libm-vs-fast-math Lanczos differences out of a comparison);
    ``normals_fn(call, n)`` supplies the random-search normals of call ``call``;
    ``nn`` the device's down-sampling index tables (see ``downsample``).
    ``proposal`` = (pred_fn, logit_min, iterations, jf_max[, local_radii[, reduce]])
    switches matching to the seeded schedule: pred_fn(prev_u8, cur_u8) gives the
    [h4][w4][3] proposal on cells of 4 * reduce input pixels (h4 = sy_in // reduce
    // 4, w4 likewise; reduce 1 by default), ``seed`` replaces the plain
    initialisation, one ``local_step`` follows per radius in local_radii, and the
    proposal's iteration count and jump maximum replace the parameters' (jf_max 0
    keeps them)."""

    def __init__(self, params: dict, pattern, normals_fn, nn=None, proposal=None):
        self.proposal = proposal
        self.prev_u8 = None
        self.p = dict(params)
        self.nn = nn
        self.pattern = np.ascontiguousarray(pattern, np.float32)
        self.normals_fn = normals_fn
        self.taps = gauss_taps(self.p["sigma"])
        self.F1 = None
        self.prev_in = None
        self.NX = self.NY = None
        self.first = True
        self.calls = 0

    def frame(self, frame_u8, up=None):
        p = self.p
        sx, sy, sxi, syi, N = p["sx"], p["sy"], p["sx_in"], p["sy_in"], p["N"]
        cur_in = np.asarray(frame_u8, np.float32)
        if up is None:
            up = cur_in if (sx == sxi and sy == syi) else upsample(cur_in, sx, sy)
        F2 = features(up, self.pattern, N)
        out = None
        if self.F1 is not None:
            n = sx * sy
            it = p["iterations"]
            nrm = np.concatenate([np.asarray(self.normals_fn(self.calls + k, n), np.float32).ravel() for k in range(it)]) \
                if it else np.zeros(2 * n, np.float32)
            first = self.first or not p["tInit"]
            if self.proposal is None:
                NX, NY, H = match(self.F1, F2, sx, sy, N, it, p["jfMax"], p["doubleProp"], first, search_dist(sx), nrm,
                                  self.NX, self.NY)
            else:
                pred_fn, logit_min, it, jf = self.proposal[:4]
                radii = self.proposal[4] if len(self.proposal) > 4 else ()
                red = self.proposal[5] if len(self.proposal) > 5 else 1
                jf = jf or p["jfMax"]
                # bm_api.cu match_impl: a cell covers 4 * reduce input pixels
                w4, h4 = sxi // red // 4, syi // red // 4
                f32 = np.float32
                scx = f32(4.0 * red) * f32(sx) / f32(sxi)
                scy = f32(4.0 * red) * f32(sy) / f32(syi)
                pred = pred_fn(self.prev_u8, frame_u8)
                NX, NY, H = seed(self.F1, F2, sx, sy, N, first, pred, w4, h4, scx, scy, logit_min, self.NX, self.NY)
                for r in radii:
                    NX, NY, H = local_step(self.F1, F2, sx, sy, N, r, NX, NY, H)
                pd = -1
                for k in range(it):
                    NX, NY, H = propagate(self.F1, F2, sx, sy, N, pd, jf, p["doubleProp"], NX, NY, H)
                    NX, NY, H = random_search(self.F1, F2, sx, sy, N, search_dist(sx),
                                              np.asarray(self.normals_fn(self.calls + k, n), np.float32).ravel(),
                                              NX, NY, H)
                    pd = -pd
            self.calls += it
            self.first = False
            self.NX, self.NY, self.H = NX, NY, H
            U, V = downsample(NX, NY, sx, sy, sxi, syi, self.taps, self.nn)
            self.U, self.V = U, V
            if p["filter"]:
                Um, Vm, Uo, Vo = refine(U, V, self.prev_in, p["fsize"], p["sEPE"], p["sI"], p["sS"])
                self.Um, self.Vm = Um, Vm
                out = (Uo, Vo)
            else:
                out = (U, V)
        self.F1 = F2
        self.prev_in = cur_in
        self.prev_u8 = np.asarray(frame_u8)
        return out
