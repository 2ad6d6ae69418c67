"""ctypes wrapper of oracle/refshim.c: the reference's own kernels, compiled from
their sources to oracle/_ref/*.cubin, launched on the GPU (TEST INFRASTRUCTURE).

Device buffers are torch CUDA tensors.  Buffers the reference reads outside their
bounds (propagation neighbours, briefmatch_cuda.cu:212-214; the median window,
util_cuda.cu:87-96) are allocated with zero guard bands on both sides, which gives
those reads the value 0 -- the same guard the engine and the oracle define.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REFSHIM_LIB = os.path.join(_HERE, "_build", "librefshim.so")
REF_DIR = os.path.join(_HERE, "_ref")
CURAND_STATE_BYTES = 48  # sizeof(curandStateXORWOW_t)

_lib = None


def available():
    return (os.path.exists(REFSHIM_LIB) and os.path.exists(os.path.join(REF_DIR, "briefmatch_cuda.cubin"))
            and os.path.exists(os.path.join(REF_DIR, "util_cuda.cubin")))


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(REFSHIM_LIB)
        u64, i, f = ctypes.c_uint64, ctypes.c_int, ctypes.c_float
        sig = {
            "rs_load": [ctypes.c_char_p, ctypes.c_char_p],
            "rs_set_pattern": [ctypes.c_void_p],
            "rs_set_kernel": [ctypes.c_void_p],
            "rs_init_random": [u64, i, i],
            "rs_binary_features": [u64, u64, i, i, i, i],
            "rs_initialize": [u64] * 7 + [i, i, i, i, i],
            "rs_propagate": [u64] * 7 + [i, i, i, i, i, i, i],
            "rs_random_search": [u64] * 8 + [i, i, f, i, i],
            "rs_cb_filter": [u64] * 7 + [f, f, f, i, i],
            "rs_filter_const": [u64, u64, i, i, i, i],
            "rs_median": [u64, u64, i, i, i, i],
            "rs_resize_lanczos": [u64, u64, i, i, i, i],
            "rs_resize_nn": [u64, u64, i, i, i, i],
            "rs_mult": [u64, f, i, i],
            "rs_convert": [u64, u64, i, i],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.restype = ctypes.c_int
            fn.argtypes = args
        L.rs_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _ck(rc):
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().rs_error().decode())


class RefKernels:
    """The reference kernel layer (CUDA_* of briefmatch_cuda.h / util_cuda.h)."""

    def __init__(self):
        import torch  # noqa: F401  (initialises the primary context the shim joins)
        _ck(lib().rs_load(os.path.join(REF_DIR, "briefmatch_cuda.cubin").encode(),
                          os.path.join(REF_DIR, "util_cuda.cubin").encode()))

    def set_pattern(self, pattern):
        buf = np.zeros(2048, np.float32)
        pattern = np.asarray(pattern, np.float32).ravel()
        buf[: pattern.size] = pattern
        _ck(lib().rs_set_pattern(buf.ctypes.data))

    def set_kernel(self, taps):
        buf = np.zeros(100, np.float32)
        taps = np.asarray(taps, np.float32).ravel()
        buf[: taps.size] = taps
        _ck(lib().rs_set_kernel(buf.ctypes.data))

    # each takes device pointers (ints), mirroring the reference launchers
    def init_random(self, state, sx, sy):
        _ck(lib().rs_init_random(state, sx, sy))

    def binary_features(self, I, F, sx, sy, N, Ns):
        _ck(lib().rs_binary_features(I, F, sx, sy, N, Ns))

    def initialize(self, F1, F2, D, NX, NY, sx, sy, first, N, Ns):
        _ck(lib().rs_initialize(0, 0, F1, F2, D, NX, NY, sx, sy, int(bool(first)), N, Ns))

    def propagate(self, F1, F2, D, NX, NY, sx, sy, pd, jf_max, double_prop, N, Ns):
        _ck(lib().rs_propagate(0, 0, F1, F2, D, NX, NY, sx, sy, pd, jf_max, int(bool(double_prop)), N, Ns))

    def random_search(self, F1, F2, D, NX, NY, state, sx, sy, dist, N, Ns):
        _ck(lib().rs_random_search(0, 0, F1, F2, D, NX, NY, state, sx, sy, dist, N, Ns))

    def cb_filter(self, Ui, Vi, Uo, Vo, Uim, Vim, I, sE2, sI2, sS2, sx, sy):
        _ck(lib().rs_cb_filter(Ui, Vi, Uo, Vo, Uim, Vim, I, sE2, sI2, sS2, sx, sy))

    def filter_const(self, Li, Lo, ks, direction, sx, sy):
        _ck(lib().rs_filter_const(Li, Lo, ks, direction, sx, sy))

    def median(self, Li, Lo, direction, fsize, sx, sy):
        _ck(lib().rs_median(Li, Lo, direction, fsize, sx, sy))

    def resize_lanczos(self, Li, Lo, sxi, syi, sxo, syo):
        _ck(lib().rs_resize_lanczos(Li, Lo, sxi, syi, sxo, syo))

    def resize_nn(self, Li, Lo, sxi, syi, sxo, syo):
        _ck(lib().rs_resize_nn(Li, Lo, sxi, syi, sxo, syo))

    def mult(self, L, m, sx, sy):
        _ck(lib().rs_mult(L, m, sx, sy))

    def convert(self, Li, Lo, sx, sy):
        _ck(lib().rs_convert(Li, Lo, sx, sy))


def guarded(torch, n, guard, dtype, device="cuda"):
    """A zero tensor with `guard` zero elements before and after an n-element body;
    returns (storage, body view)."""
    store = torch.zeros(n + 2 * guard, dtype=dtype, device=device)
    return store, store[guard:guard + n]


class RefPipeline:
    """OFPipeline::processFrame + BriefMatch::match/downsample/process
    (of_pipeline.cpp:296-333, briefmatch.cpp:248-352) driven through the
    reference's own kernels, for timing the reference build on the GPU.

    Frames are float input-resolution device tensors (the reference uploads
    float, of_pipeline.cpp:297).  The first frame primes (descriptors only), as
    the engine does; later frames run the full pair.  Buffers the reference
    reads out of bounds carry zero guard bands."""

    def __init__(self, torch, params: dict, pattern, taps):
        self.t = torch
        self.k = RefKernels()
        p = self.p = dict(params)
        self.k.set_pattern(pattern)
        self.k.set_kernel(taps)
        self.P = len(taps)
        sx, sy, sxi, syi = p["sx"], p["sy"], p["sx_in"], p["sy_in"]
        n, ni = sx * sy, sxi * syi
        self.ns = (p["N"] + 31) // 32
        g = (p["jfMax"] + 1) * sx + p["jfMax"]
        gm = (p["fsize"] // 2 + 1) * sxi + p["fsize"]
        z = lambda cnt, dt=torch.float32: torch.zeros(cnt, dtype=dt, device="cuda")
        self.L = z(n)
        self.F = [z(n * self.ns, torch.int32), z(n * self.ns, torch.int32)]
        self.D = z(n)
        self._nx_store, self.NX = guarded(torch, n, g, torch.int16)
        self._ny_store, self.NY = guarded(torch, n, g, torch.int16)
        self.XF, self.YF, self.tmp = z(n), z(n), z(n)
        self.state = z(n * CURAND_STATE_BYTES, torch.uint8)
        self._xi, self.XI = guarded(torch, ni, gm, torch.float32)
        self._yi, self.YI = guarded(torch, ni, gm, torch.float32)
        self._ti, self.TI = guarded(torch, ni, gm, torch.float32)
        self.XM, self.YM, self.XO, self.YO = z(ni), z(ni), z(ni), z(ni)
        self.k.init_random(self.state.data_ptr(), sx, sy)
        self.dist = float(np.sqrt(np.ceil(np.float32(sx) * np.float32(0.5) / np.float32(3.0)), dtype=np.float32))
        self.first = True
        self.primed = False
        self.prev_in = None

    def frame(self, d_in):
        p, k = self.p, self.k
        sx, sy, sxi, syi, N, ns = p["sx"], p["sy"], p["sx_in"], p["sy_in"], p["N"], self.ns
        F1, F2 = self.F
        if sx != sxi or sy != syi:
            k.resize_lanczos(d_in.data_ptr(), self.L.data_ptr(), sxi, syi, sx, sy)
            L = self.L
        else:
            L = d_in
        k.binary_features(L.data_ptr(), F2.data_ptr(), sx, sy, N, ns)
        if self.primed:
            k.initialize(F1.data_ptr(), F2.data_ptr(), self.D.data_ptr(), self.NX.data_ptr(), self.NY.data_ptr(), sx, sy,
                         self.first or not p["tInit"], N, ns)
            pd = -1
            for _ in range(p["iterations"]):
                k.propagate(F1.data_ptr(), F2.data_ptr(), self.D.data_ptr(), self.NX.data_ptr(), self.NY.data_ptr(), sx, sy,
                            pd, p["jfMax"], p["doubleProp"], N, ns)
                k.random_search(F1.data_ptr(), F2.data_ptr(), self.D.data_ptr(), self.NX.data_ptr(), self.NY.data_ptr(),
                                self.state.data_ptr(), sx, sy, self.dist, N, ns)
                pd = -pd
            self.first = False
            k.convert(self.NX.data_ptr(), self.XF.data_ptr(), sx, sy)
            k.convert(self.NY.data_ptr(), self.YF.data_ptr(), sx, sy)
            if sx != sxi or sy != syi:
                for F in (self.XF, self.YF):
                    k.filter_const(F.data_ptr(), self.tmp.data_ptr(), self.P, 1, sx, sy)
                    k.filter_const(self.tmp.data_ptr(), F.data_ptr(), self.P, 0, sx, sy)
                k.resize_nn(self.XF.data_ptr(), self.XI.data_ptr(), sx, sy, sxi, syi)
                k.resize_nn(self.YF.data_ptr(), self.YI.data_ptr(), sx, sy, sxi, syi)
                k.mult(self.XI.data_ptr(), float(np.float32(sxi) / np.float32(sx)), sxi, syi)
                k.mult(self.YI.data_ptr(), float(np.float32(syi) / np.float32(sy)), sxi, syi)
            if p["filter"]:
                k.median(self.XI.data_ptr(), self.TI.data_ptr(), 1, p["fsize"], sxi, syi)
                k.median(self.TI.data_ptr(), self.XM.data_ptr(), 0, p["fsize"], sxi, syi)
                k.median(self.YI.data_ptr(), self.TI.data_ptr(), 1, p["fsize"], sxi, syi)
                k.median(self.TI.data_ptr(), self.YM.data_ptr(), 0, p["fsize"], sxi, syi)
                k.cb_filter(self.XI.data_ptr(), self.YI.data_ptr(), self.XO.data_ptr(), self.YO.data_ptr(),
                            self.XM.data_ptr(), self.YM.data_ptr(), self.prev_in.data_ptr(),
                            p["sEPE"] * p["sEPE"], p["sI"] * p["sI"], p["sS"] * p["sS"], sxi, syi)
        self.primed = True
        self.F.reverse()
        self.prev_in = d_in
