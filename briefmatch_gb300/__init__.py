"""briefmatch_gb300 -- GB300-native BriefMatch dense optical flow.

Python view of the engine's C ABI (include/briefmatch_gb300.h), loaded with
ctypes from the in-tree library briefmatch_gb300/_lib/libbriefmatch_gb300.so.
There is no CPU fallback: importing the engine without its compiled library
raises.  Device buffers handed to the stage functions are raw CUDA pointers
(for example ``tensor.data_ptr()`` of a torch CUDA tensor).

The classes mirror the reference's host API:
  BMParams    briefmatch.h:65-89
  BriefMatch  briefmatch.h:108-155 (setup/match/downsample/process/swap/convert)
  FlowEngine  OFPipeline::processFrame (of_pipeline.cpp:241-387) over 8-bit frames
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libbriefmatch_gb300.so")

BM_PATCH_MAX = 2048
BM_MAX_MEDIAN = 47
BM_CONST_KERNEL_SIZE = 100

BM_OK, BM_ERR_INVALID, BM_ERR_LIMIT, BM_ERR_CUDA, BM_ERR_STATE, BM_ERR_NOMEM, BM_ERR_TIMEOUT, BM_ERR_IO = range(8)
BM_RNG_XORWOW, BM_RNG_PHILOX = 0, 1
(BM_BUF_FEAT1, BM_BUF_FEAT2, BM_BUF_FLOW, BM_BUF_COST, BM_BUF_UP, BM_BUF_FLOW_IN, BM_BUF_FLOW_MED,
 BM_BUF_FLOW_OUT, BM_BUF_FRAME, BM_BUF_FRAME_PREV) = range(10)


class BriefMatchException(RuntimeError):
    """Parameter-limit and state errors (briefmatch.h:91-106)."""


class CudaException(RuntimeError):
    """CUDA runtime errors (util_cuda.h:85-100)."""


class bm_kernel_stat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("launches", ctypes.c_uint64), ("ms", ctypes.c_double)]


class bm_params(ctypes.Structure):
    _fields_ = [
        ("sx", ctypes.c_uint32), ("sy", ctypes.c_uint32), ("sx_in", ctypes.c_uint32), ("sy_in", ctypes.c_uint32),
        ("N", ctypes.c_uint32), ("iterations", ctypes.c_uint32), ("jfMax", ctypes.c_uint32), ("P", ctypes.c_uint32),
        ("fsize", ctypes.c_uint32),
        ("patchArea", ctypes.c_float), ("sigma", ctypes.c_float), ("sEPE", ctypes.c_float), ("sI", ctypes.c_float),
        ("sS", ctypes.c_float), ("maxmot", ctypes.c_float),
        ("doubleProp", ctypes.c_int32), ("filter", ctypes.c_int32), ("tInit", ctypes.c_int32),
        ("rng", ctypes.c_uint32), ("seed", ctypes.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def _declare(lib):
    P = ctypes.POINTER
    c = ctypes
    sig = {
        "bm_params_default": (c.c_int, [P(bm_params)]),
        "bm_params_derive": (c.c_int, [P(bm_params), c.c_uint32, c.c_uint32, c.c_float, c.c_float, c.c_float,
                                       c.c_float, c.c_float, c.c_float]),
        "bm_make_pattern": (c.c_int, [P(bm_params), c.c_uint64, P(c.c_float)]),
        "bm_gauss_taps": (c.c_int, [c.c_float, P(c.c_float), P(c.c_uint32)]),
        "bm_create": (c.c_int, [P(bm_params), P(c.c_void_p)]),
        "bm_destroy": (c.c_int, [c.c_void_p]),
        "bm_get_params": (c.c_int, [c.c_void_p, P(bm_params)]),
        "bm_set_stream": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_synchronize": (c.c_int, [c.c_void_p]),
        "bm_set_pattern": (c.c_int, [c.c_void_p, P(c.c_float), c.c_uint32]),
        "bm_buffer": (c.c_int, [c.c_void_p, c.c_int, P(c.c_void_p), P(c.c_size_t)]),
        "bm_feature_stride": (c.c_uint32, [c.c_void_p]),
        "bm_read_buffer": (c.c_int, [c.c_void_p, c.c_int, c.c_void_p, c.c_size_t, c.c_int]),
        "bm_write_buffer": (c.c_int, [c.c_void_p, c.c_int, c.c_void_p, c.c_size_t, c.c_int]),
        "bm_upsample": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_upsample_u8": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_features": (c.c_int, [c.c_void_p, c.c_void_p, c.c_int]),
        "bm_initialize": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_propagate": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_random_search": (c.c_int, [c.c_void_p]),
        "bm_match": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_downsample": (c.c_int, [c.c_void_p]),
        "bm_process": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_swap": (c.c_int, [c.c_void_p]),
        "bm_convert": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_colors": (c.c_int, [c.c_void_p, c.c_void_p, c.c_int]),
        "bm_flow_colors": (c.c_int, [c.c_void_p, c.c_void_p, c.c_uint32, c.c_uint32, c.c_float, c.c_void_p,
                                     c.c_void_p]),
        "bm_export_field": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_import_field": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_normals": (c.c_int, [c.c_void_p, c.c_uint64, c.c_void_p]),
        "bm_nn_indices": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_rng_position": (c.c_int, [c.c_void_p, P(c.c_uint64)]),
        "bm_set_rng_position": (c.c_int, [c.c_void_p, c.c_uint64]),
        "bm_frame": (c.c_int, [c.c_void_p, c.c_void_p, c.c_int, c.c_void_p, c.c_void_p, c.c_int]),
        "bm_reset_sequence": (c.c_int, [c.c_void_p]),
        "bm_launch_count": (c.c_uint64, [c.c_void_p]),
        "bm_profile_enable": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_profile_reset": (c.c_int, [c.c_void_p]),
        "bm_profile_read": (c.c_int, [c.c_void_p, c.c_void_p, c.c_uint32, P(c.c_uint32)]),
        "bm_set_proposal": (c.c_int, [c.c_void_p, c.c_void_p, c.c_float, c.c_uint32, c.c_uint32]),
        "bm_set_proposal_stream": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_set_proposal_reduce": (c.c_int, [c.c_void_p, c.c_uint32]),
        "bm_set_pipelined": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_set_local_steps": (c.c_int, [c.c_void_p, c.c_uint32, c.c_uint32]),
        "bm_local_step": (c.c_int, [c.c_void_p, c.c_uint32]),
        "bm_batch_set_local_steps": (c.c_int, [c.c_void_p, c.c_uint32, c.c_uint32]),
        "bm_join": (c.c_int, [c.c_void_p]),
        "bm_batch_set_proposal": (c.c_int, [c.c_void_p, c.c_void_p, c.c_float, c.c_uint32, c.c_uint32]),
        "bm_batch_set_proposal_reduce": (c.c_int, [c.c_void_p, c.c_uint32]),
        "bm_seed": (c.c_int, [c.c_void_p, c.c_int, c.c_void_p, c.c_uint32, c.c_uint32, c.c_float]),
        "bm_refine_noalloc": (c.c_int, [c.c_void_p, c.c_void_p, c.c_void_p, c.c_void_p, c.c_void_p, c.c_uint32,
                                        c.c_uint32, c.c_uint32, c.c_float, c.c_float, c.c_float, c.c_void_p]),
        "bm_refine_noalloc_max_pixels": (c.c_uint64, []),
        "bm_batch_create": (c.c_int, [c.c_void_p, c.c_uint32, P(c.c_void_p)]),
        "bm_batch_destroy": (c.c_int, [c.c_void_p]),
        "bm_batch_count": (c.c_uint32, [c.c_void_p]),
        "bm_batch_set_stream": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_batch_set_pattern": (c.c_int, [c.c_void_p, c.c_uint32, c.c_void_p, c.c_uint32]),
        "bm_batch_frames_bytes": (c.c_size_t, [c.c_void_p]),
        "bm_batch_flows_bytes": (c.c_size_t, [c.c_void_p]),
        "bm_batch_frame_ptr": (c.c_int, [c.c_void_p, c.c_uint32, c.c_uint32, P(c.c_void_p)]),
        "bm_batch_load_frames": (c.c_int, [c.c_void_p, c.c_void_p, c.c_size_t, c.c_int]),
        "bm_batch_read_flows": (c.c_int, [c.c_void_p, c.c_void_p, c.c_size_t, c.c_int]),
        "bm_batch_flow_ptr": (c.c_int, [c.c_void_p, c.c_uint32, P(c.c_void_p), P(c.c_void_p)]),
        "bm_batch_set_schedule": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_batch_get_schedule": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_batch_run": (c.c_int, [c.c_void_p]),
        "bm_batch_synchronize": (c.c_int, [c.c_void_p]),
        "bm_batch_launch_count": (c.c_uint64, [c.c_void_p]),
        "bm_batch_autotune": (c.c_int, [c.c_void_p, c.c_char_p, c.c_int, c.c_char_p, c.c_size_t]),
        "bm_selftest_barrier": (c.c_int, [c.c_uint32, c.c_uint32, c.c_uint64, P(c.c_int)]),
        "bm_debug_fail_alloc": (None, [c.c_uint64]),
        "bm_debug_alloc_count": (c.c_uint64, []),
        "bm_debug_live_allocs": (c.c_int64, []),
        "bm_debug_guard_bands": (None, [c.c_int]),
        "bm_debug_check_guards": (c.c_int, [P(c.c_uint64)]),
        "bm_last_error": (c.c_char_p, []),
        "bm_version": (c.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "briefmatch_gb300: engine library missing at %s; run __graft_entry__.build() "
                "(the engine has no CPU fallback)" % LIB_PATH)
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def check(status):
    if status == BM_OK:
        return
    msg = lib().bm_last_error().decode(errors="replace")
    if status in (BM_ERR_LIMIT, BM_ERR_STATE, BM_ERR_INVALID):
        raise BriefMatchException(msg)
    raise CudaException("status %d: %s" % (status, msg))


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class BMParams:
    """BMParams (briefmatch.h:65-89) with OFPipeline's derivation (of_pipeline.cpp:178-190)."""

    def __init__(self, **kw):
        self._p = bm_params()
        check(lib().bm_params_default(ctypes.byref(self._p)))
        for k, v in kw.items():
            setattr(self._p, k, v)

    @classmethod
    def derive(cls, width, height, ux=0.0, uy=0.0, patch_radius=3.0, sigma_downsampling=0.025, median_size=1.0,
               range_spatial=0.85, **kw):
        """Parameters for a width x height input as OFPipeline::setParams derives them
        from the command-line percentages (defaults of_pipeline.cpp:94-95)."""
        self = cls(**kw)
        check(lib().bm_params_derive(ctypes.byref(self._p), width, height, ux, uy, patch_radius, sigma_downsampling,
                                     median_size, range_spatial))
        return self

    def __getattr__(self, k):
        if k.startswith("_"):
            raise AttributeError(k)
        return getattr(self._p, k)

    def __setattr__(self, k, v):
        if k == "_p":
            object.__setattr__(self, k, v)
        else:
            setattr(self._p, k, v)

    def struct(self):
        return self._p

    def as_dict(self):
        return self._p.as_dict()

    def make_pattern(self, seed=0):
        out = np.zeros(4 * self._p.N, np.float32)
        check(lib().bm_make_pattern(ctypes.byref(self._p), seed, _fptr(out)))
        return out

    def gauss_taps(self):
        out = np.zeros(BM_CONST_KERNEL_SIZE, np.float32)
        P = ctypes.c_uint32(0)
        check(lib().bm_gauss_taps(self._p.sigma, _fptr(out), ctypes.byref(P)))
        return out[: P.value].copy()

    def search_dist(self):
        """Random-search radius, briefmatch.cpp:271."""
        return float(np.sqrt(np.ceil(np.float32(self._p.sx) * np.float32(0.5) / np.float32(3.0)), dtype=np.float32))


class BriefMatch:
    """Engine context over the C ABI; method names follow briefmatch.h:108-135."""

    def __init__(self, params: BMParams | None = None):
        self.params = params or BMParams()
        self._ctx = ctypes.c_void_p(None)

    # lifecycle -------------------------------------------------------------
    def setup(self):
        if self._ctx:
            return
        check(lib().bm_create(ctypes.byref(self.params.struct()), ctypes.byref(self._ctx)))
        p = bm_params()
        check(lib().bm_get_params(self._ctx, ctypes.byref(p)))
        self.params.P = p.P

    def clean(self):
        if self._ctx:
            lib().bm_destroy(self._ctx)
            self._ctx = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.clean()
        except Exception:
            pass

    def isSetup(self):
        return bool(self._ctx)

    @property
    def ctx(self):
        if not self._ctx:
            raise BriefMatchException("BriefMatch is not initialized before use.")
        return self._ctx

    # configuration -------------------------------------------------------------
    def set_stream(self, stream_ptr):
        check(lib().bm_set_stream(self.ctx, ctypes.c_void_p(stream_ptr)))

    def synchronize(self):
        check(lib().bm_synchronize(self.ctx))

    def set_pattern(self, pattern):
        pat = np.ascontiguousarray(pattern, dtype=np.float32)
        check(lib().bm_set_pattern(self.ctx, _fptr(pat), pat.size))

    def buffer(self, which):
        ptr = ctypes.c_void_p(None)
        nbytes = ctypes.c_size_t(0)
        check(lib().bm_buffer(self.ctx, which, ctypes.byref(ptr), ctypes.byref(nbytes)))
        return ptr.value, nbytes.value

    def read_buffer(self, which, dtype, count=None):
        """Host copy of a context buffer as a numpy array."""
        _, nbytes = self.buffer(which)
        dt = np.dtype(dtype)
        count = nbytes // dt.itemsize if count is None else count
        out = np.empty(count, dt)
        check(lib().bm_read_buffer(self.ctx, which, out.ctypes.data, out.nbytes, 0))
        return out

    def write_buffer(self, which, array):
        a = np.ascontiguousarray(array)
        check(lib().bm_write_buffer(self.ctx, which, a.ctypes.data, a.nbytes, 0))

    def feature_stride(self):
        return lib().bm_feature_stride(self.ctx)

    # stages ---------------------------------------------------------------
    def upsample(self, d_in, d_out):
        check(lib().bm_upsample(self.ctx, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out)))

    def upsample_u8(self, d_in, d_out):
        check(lib().bm_upsample_u8(self.ctx, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out)))

    def features(self, d_up, slot):
        check(lib().bm_features(self.ctx, ctypes.c_void_p(d_up), slot))

    def initialize(self, first):
        check(lib().bm_initialize(self.ctx, int(bool(first))))

    def propagate(self, pd):
        check(lib().bm_propagate(self.ctx, pd))

    def random_search(self):
        check(lib().bm_random_search(self.ctx))

    def match(self, d_im1, d_im2):
        check(lib().bm_match(self.ctx, ctypes.c_void_p(d_im1 or 0), ctypes.c_void_p(d_im2)))

    def downsample(self):
        check(lib().bm_downsample(self.ctx))

    def process(self, d_prev_in):
        check(lib().bm_process(self.ctx, ctypes.c_void_p(d_prev_in)))

    def swap(self):
        check(lib().bm_swap(self.ctx))

    def convert(self):
        n = self.params.sx_in * self.params.sy_in
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        check(lib().bm_convert(self.ctx, u.ctypes.data, v.ctypes.data))
        return u.reshape(self.params.sy_in, self.params.sx_in), v.reshape(self.params.sy_in, self.params.sx_in)

    def compute_colors(self, d_rgb=None):
        """BriefMatch::computeColors on the GPU: the output field colour-coded, R G B
        bytes per pixel.  With a device pointer the bytes go there; else an
        [sy_in][sx_in][3] uint8 array is returned."""
        if d_rgb is not None:
            check(lib().bm_colors(self.ctx, ctypes.c_void_p(d_rgb), 1))
            return None
        out = np.empty((self.params.sy_in, self.params.sx_in, 3), np.uint8)
        check(lib().bm_colors(self.ctx, out.ctypes.data, 0))
        return out

    def export_field(self, d_nx, d_ny, d_dist):
        check(lib().bm_export_field(self.ctx, ctypes.c_void_p(d_nx or 0), ctypes.c_void_p(d_ny or 0),
                                    ctypes.c_void_p(d_dist or 0)))

    def import_field(self, d_nx, d_ny, d_cost):
        check(lib().bm_import_field(self.ctx, ctypes.c_void_p(d_nx), ctypes.c_void_p(d_ny),
                                    ctypes.c_void_p(d_cost or 0)))

    def normals(self, call, d_out):
        check(lib().bm_normals(self.ctx, call, ctypes.c_void_p(d_out)))

    def nn_indices(self):
        """resizeNN source column/row per input column/row (util_cuda.cu:165-166)."""
        xs = np.empty(self.params.sx_in, np.uint32)
        ys = np.empty(self.params.sy_in, np.uint32)
        check(lib().bm_nn_indices(self.ctx, xs.ctypes.data, ys.ctypes.data))
        return xs, ys

    def rng_position(self):
        v = ctypes.c_uint64(0)
        check(lib().bm_rng_position(self.ctx, ctypes.byref(v)))
        return v.value

    def set_rng_position(self, calls):
        check(lib().bm_set_rng_position(self.ctx, calls))

    def frame(self, frame_ptr, on_device, u_ptr=None, v_ptr=None, out_on_device=True):
        check(lib().bm_frame(self.ctx, ctypes.c_void_p(frame_ptr), int(bool(on_device)), ctypes.c_void_p(u_ptr or 0),
                             ctypes.c_void_p(v_ptr or 0), int(bool(out_on_device))))

    def reset_sequence(self):
        check(lib().bm_reset_sequence(self.ctx))

    def set_pipelined(self, on=True):
        """Overlap each pair's refinement with the next frame (bm_set_pipelined)."""
        check(lib().bm_set_pipelined(self.ctx, int(bool(on))))

    def join(self):
        """The context stream waits for the pipelined refinement queued so far."""
        check(lib().bm_join(self.ctx))

    def launch_count(self):
        return int(lib().bm_launch_count(self.ctx))

    def profile(self, on=True):
        check(lib().bm_profile_enable(self.ctx, int(bool(on))))

    def profile_reset(self):
        check(lib().bm_profile_reset(self.ctx))

    def profile_read(self):
        """{kernel name: (launches, total ms)} since the last reset (synchronises)."""
        n = ctypes.c_uint32(0)
        check(lib().bm_profile_read(self.ctx, None, 0, ctypes.byref(n)))
        arr = (bm_kernel_stat * max(1, n.value))()
        check(lib().bm_profile_read(self.ctx, arr, n.value, ctypes.byref(n)))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].ms)) for i in range(n.value)}


class FlowEngine(BriefMatch):
    """Frame-at-a-time flow over 8-bit host frames: OFPipeline::processFrame
    (of_pipeline.cpp:241-387) without file I/O.  The first frame primes the
    context and yields zeros; each later frame yields the flow from the previous
    frame to it, sampled on the previous frame's grid, as (u, v) float32 arrays."""

    def __init__(self, params: BMParams):
        super().__init__(params)
        self.setup()

    def process_frame(self, frame_u8):
        f = np.ascontiguousarray(frame_u8, dtype=np.uint8)
        p = self.params
        if f.shape != (p.sy_in, p.sx_in):
            raise BriefMatchException("frame shape %s does not match %dx%d" % (f.shape, p.sx_in, p.sy_in))
        u = np.empty((p.sy_in, p.sx_in), np.float32)
        v = np.empty((p.sy_in, p.sx_in), np.float32)
        self.frame(f.ctypes.data, False, u.ctypes.data, v.ctypes.data, out_on_device=False)
        return u, v


class bm_batch_schedule(ctypes.Structure):
    _fields_ = [("persistent", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32), ("snake", ctypes.c_uint32),
                ("use_graph", ctypes.c_uint32), ("spin_limit", ctypes.c_uint64), ("wave_bytes", ctypes.c_uint64),
                ("per_pair", ctypes.c_uint32), ("streams", ctypes.c_uint32)]


class Batch:
    """Many frame pairs of uneven size computed together (bm_batch_* in the C ABI).

    ``params`` is one BMParams per pair (all with the same N, iterations, jfMax,
    doubleProp, filter and random stream).  Pair i's result equals what a fresh
    FlowEngine computes for its two frames."""

    def __init__(self, params):
        arr = (bm_params * len(params))(*[p.struct() for p in params])
        self.params = list(params)
        self._b = ctypes.c_void_p(None)
        check(lib().bm_batch_create(arr, len(params), ctypes.byref(self._b)))
        self.frames_bytes = lib().bm_batch_frames_bytes(self._b)
        self.flows_bytes = lib().bm_batch_flows_bytes(self._b)

    def close(self):
        if self._b:
            lib().bm_batch_destroy(self._b)
            self._b = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        check(lib().bm_batch_set_stream(self._b, ctypes.c_void_p(stream_ptr)))

    def set_pattern(self, pair, pattern):
        pat = np.ascontiguousarray(pattern, np.float32)
        check(lib().bm_batch_set_pattern(self._b, pair, pat.ctypes.data, pat.size))

    def pack_frames(self, pairs_of_frames):
        """Host packing of [(frame0, frame1), ...] in the batch's frame layout."""
        parts = []
        for (f0, f1), p in zip(pairs_of_frames, self.params):
            for f in (f0, f1):
                f = np.ascontiguousarray(f, np.uint8)
                assert f.shape == (p.sy_in, p.sx_in)
                parts.append(f.ravel())
        out = np.concatenate(parts)
        assert out.nbytes == self.frames_bytes
        return out

    def load_frames(self, packed, on_device=False):
        ptr = packed if isinstance(packed, int) else packed.ctypes.data
        check(lib().bm_batch_load_frames(self._b, ctypes.c_void_p(ptr), self.frames_bytes, int(bool(on_device))))

    def frame_ptr(self, pair, which):
        p = ctypes.c_void_p(None)
        check(lib().bm_batch_frame_ptr(self._b, pair, which, ctypes.byref(p)))
        return p.value

    def run(self):
        check(lib().bm_batch_run(self._b))

    def synchronize(self):
        check(lib().bm_batch_synchronize(self._b))

    def read_flows(self):
        out = np.empty(self.flows_bytes // 4, np.float32)
        check(lib().bm_batch_read_flows(self._b, out.ctypes.data, self.flows_bytes, 0))
        res, k = [], 0
        for p in self.params:
            n = p.sx_in * p.sy_in
            res.append((out[k:k + n].reshape(p.sy_in, p.sx_in), out[k + n:k + 2 * n].reshape(p.sy_in, p.sx_in)))
            k += 2 * n
        return res

    def read_flows_into(self, ptr, on_device):
        check(lib().bm_batch_read_flows(self._b, ctypes.c_void_p(ptr), self.flows_bytes, int(bool(on_device))))

    def schedule(self):
        s = bm_batch_schedule()
        check(lib().bm_batch_get_schedule(self._b, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def set_schedule(self, **kw):
        s = bm_batch_schedule()
        check(lib().bm_batch_get_schedule(self._b, ctypes.byref(s)))
        for k, v in kw.items():
            setattr(s, k, v)
        check(lib().bm_batch_set_schedule(self._b, ctypes.byref(s)))

    def autotune(self, cache_path=None, reps=3):
        buf = ctypes.create_string_buffer(2048)
        check(lib().bm_batch_autotune(self._b, cache_path.encode() if cache_path else None, reps, buf, 2048))
        return buf.value.decode()

    def launch_count(self):
        return int(lib().bm_batch_launch_count(self._b))

    def set_local_steps(self, count, first_radius=2):
        """Local refinement steps after each pair's seeded initialisation."""
        check(lib().bm_batch_set_local_steps(self._b, count, first_radius))

    def set_proposal(self, net, conf_threshold=0.5, iterations=1, jf_max=16):
        """Seed every pair with a ProposalNet (None detaches); see bm_batch_set_proposal."""
        check(lib().bm_batch_set_proposal(self._b, net.handle if net is not None else None, conf_threshold,
                                          iterations, jf_max))

    def set_proposal_reduce(self, reduce):
        """The network's input reduction for every pair (bm_batch_set_proposal_reduce)."""
        check(lib().bm_batch_set_proposal_reduce(self._b, reduce))


def set_proposal_stream(engine, side=True):
    """Whether the context runs the proposal network on its own side stream or on the
    context stream (bm_set_proposal_stream; the context stream is the default)."""
    check(lib().bm_set_proposal_stream(engine.ctx, int(bool(side))))


def set_proposal(engine, net, conf_threshold=0.5, iterations=1, jf_max=16):
    """Attach a ProposalNet (or None) to a BriefMatch context (bm_set_proposal)."""
    check(lib().bm_set_proposal(engine.ctx, net.handle if net is not None else None, conf_threshold, iterations,
                                jf_max))


def set_proposal_reduce(engine, reduce):
    """Cells of 4 * reduce input pixels for the context's proposal network: the
    network sees the frames reduced by `reduce` (bm_set_proposal_reduce)."""
    check(lib().bm_set_proposal_reduce(engine.ctx, reduce))


def set_local_steps(engine, count, first_radius=2):
    """Local refinement steps after the seeded initialisation (bm_set_local_steps)."""
    check(lib().bm_set_local_steps(engine.ctx, count, first_radius))


def local_step(engine, radius):
    """One local refinement step on the current field (bm_local_step)."""
    check(lib().bm_local_step(engine.ctx, radius))


def seed(engine, first, d_pred, w4, h4, conf_threshold=0.5):
    """Seeded initialisation from a [h4][w4][3] device prediction (bm_seed)."""
    check(lib().bm_seed(engine.ctx, int(bool(first)), ctypes.c_void_p(d_pred), w4, h4, conf_threshold))


def selftest_barrier(blocks, expect, spin_limit):
    """(status, timed_out) of the bounded grid-barrier self-test."""
    t = ctypes.c_int(0)
    st = lib().bm_selftest_barrier(blocks, expect, spin_limit, ctypes.byref(t))
    return st, t.value


def refine_noalloc(d_u, d_v, d_guide, d_uo, d_vo, width, height, fsize, sEPE, sI, sS, stream=0):
    """Median + cross-trilateral refinement on caller-owned device buffers without
    any device allocation (fixed scratch in the library; see bm_refine_noalloc)."""
    check(lib().bm_refine_noalloc(ctypes.c_void_p(d_u), ctypes.c_void_p(d_v), ctypes.c_void_p(d_guide),
                                  ctypes.c_void_p(d_uo), ctypes.c_void_p(d_vo), width, height, fsize, sEPE, sI, sS,
                                  ctypes.c_void_p(stream)))


def flow_colors(d_u, d_v, width, height, max_motion, d_rgb, stream=0):
    """Colour coding of any device field (bm_flow_colors), normalised by max_motion."""
    check(lib().bm_flow_colors(ctypes.c_void_p(d_u), ctypes.c_void_p(d_v), width, height, max_motion,
                               ctypes.c_void_p(d_rgb), ctypes.c_void_p(stream)))


def debug_fail_alloc(k):
    """Test hook: the k-th device allocation from now on fails (0 disables)."""
    lib().bm_debug_fail_alloc(k)


def debug_live_allocs():
    return int(lib().bm_debug_live_allocs())


def debug_guard_bands(on):
    """Test hook: guard bands around every device buffer allocated while on."""
    lib().bm_debug_guard_bands(int(bool(on)))


def debug_check_guards():
    """Number of guarded buffers checked; raises if a guard band was overwritten."""
    n = ctypes.c_uint64(0)
    check(lib().bm_debug_check_guards(ctypes.byref(n)))
    return n.value


def version():
    return lib().bm_version().decode()
