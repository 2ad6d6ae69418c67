"""The learned flow proposal over the engine's C ABI (bm_net_*).

ProposalNet wraps the 6-layer BF16 convolutional network: preparing inputs from
8-bit frames, the forward pass and a training step (forward, loss, backward and Adam
on the tensor-core kernels).  Parameters save and load as a flat float32 file.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import check, lib

_declared = False


def _declare():
    global _declared
    if _declared:
        return
    L = lib()
    c = ctypes
    sig = {
        "bm_net_param_count": (c.c_size_t, []),
        "bm_net_create": (c.c_int, [c.c_uint32, c.c_uint32, c.c_uint32, c.POINTER(c.c_void_p)]),
        "bm_net_destroy": (c.c_int, [c.c_void_p]),
        "bm_net_set_params": (c.c_int, [c.c_void_p, c.c_void_p, c.c_size_t]),
        "bm_net_get_params": (c.c_int, [c.c_void_p, c.c_void_p, c.c_size_t]),
        "bm_net_prepare": (c.c_int, [c.c_void_p, c.c_uint32, c.c_void_p, c.c_void_p, c.c_uint32, c.c_uint32, c.c_void_p]),
        "bm_net_prepare_reduced": (c.c_int, [c.c_void_p, c.c_uint32, c.c_void_p, c.c_void_p, c.c_uint32, c.c_uint32,
                                             c.c_uint32, c.c_void_p]),
        "bm_net_set_input": (c.c_int, [c.c_void_p, c.c_void_p, c.c_uint32, c.c_uint32, c.c_uint32, c.c_void_p]),
        "bm_net_forward": (c.c_int, [c.c_void_p, c.c_uint32, c.c_uint32, c.c_uint32, c.c_void_p, c.c_void_p]),
        "bm_net_train_step": (c.c_int, [c.c_void_p, c.c_uint32, c.c_uint32, c.c_uint32, c.c_void_p, c.c_float,
                                        c.c_void_p, c.c_void_p, c.c_void_p]),
        "bm_net_set_umma": (c.c_int, [c.c_void_p, c.c_int]),
        "bm_net_umma": (c.c_int, [c.c_void_p]),
        "bm_net_check": (c.c_int, [c.c_void_p, c.c_void_p]),
        "bm_net_snapshot": (c.c_int, [c.c_void_p, c.c_uint32, c.c_void_p]),
        "bm_net_restore": (c.c_int, [c.c_void_p, c.c_uint32, c.c_void_p]),
        "bm_net_fused_ctas": (c.c_int, [c.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _declared = True


def flops_per_pixel():
    """Multiply-add FLOPs of one forward pass per quarter-resolution pixel (real
    channels: 3x3 taps, five 32 -> 32 (the first on both frames' 4x4 pixel blocks),
    32 -> 3)."""
    cin = [32, 32, 32, 32, 32, 32]
    cout = [32, 32, 32, 32, 32, 3]
    return sum(2 * 9 * a * b for a, b in zip(cin, cout))


def param_count():
    _declare()
    return int(lib().bm_net_param_count())


class ProposalNet:
    def __init__(self, max_batch, max_h4, max_w4):
        _declare()
        self._n = ctypes.c_void_p(None)
        check(lib().bm_net_create(max_batch, max_h4, max_w4, ctypes.byref(self._n)))
        self.nparam = param_count()

    def close(self):
        if self._n:
            lib().bm_net_destroy(self._n)
            self._n = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._n

    def params(self):
        out = np.empty(self.nparam, np.float32)
        check(lib().bm_net_get_params(self._n, out.ctypes.data, out.size))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().bm_net_set_params(self._n, p.ctypes.data, p.size))

    def save(self, path):
        self.params().tofile(path)

    def load(self, path):
        self.set_params(np.fromfile(path, np.float32))

    def prepare(self, b, d_f0, d_f1, W, H, stream=0, reduce=1):
        """Input image b from two 8-bit W x H device frames, reduced by `reduce`
        (bm_net_prepare_reduced): ((W // reduce) // 4) x ((H // reduce) // 4) cells."""
        check(lib().bm_net_prepare_reduced(self._n, b, ctypes.c_void_p(d_f0), ctypes.c_void_p(d_f1), W, H, reduce,
                                           ctypes.c_void_p(stream)))

    def set_input(self, d_in_bf16, B, h, w, stream=0):
        check(lib().bm_net_set_input(self._n, ctypes.c_void_p(d_in_bf16), B, h, w, ctypes.c_void_p(stream)))

    def forward(self, B, h, w, d_out=0, stream=0):
        check(lib().bm_net_forward(self._n, B, h, w, ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))

    def set_umma(self, mode=1):
        """Convolution path (bm_net_set_umma): 1 (or True; the default) tcgen05 per layer,
        2 the fused cooperative tcgen05 forward, 0 (or False) mma.sync."""
        mode = 1 if mode is True else 0 if mode is False else int(mode)
        check(lib().bm_net_set_umma(self._n, mode))

    @property
    def umma(self):
        """The convolution path in use: 2, 1 or 0 (see set_umma)."""
        return int(lib().bm_net_umma(self._n))

    @property
    def fused_ctas(self):
        """Co-resident CTAs of the fused forward launch on this device."""
        return int(lib().bm_net_fused_ctas(self._n))

    def check(self, stream=0):
        """Raises if a tensor-core layer's bounded wait gave up (bm_net_check)."""
        check(lib().bm_net_check(self._n, ctypes.c_void_p(stream)))

    def snapshot(self, slot=0, stream=0):
        """Copy the training state into snapshot slot 0 or 1 (bm_net_snapshot)."""
        check(lib().bm_net_snapshot(self._n, slot, ctypes.c_void_p(stream)))

    def restore(self, slot=0, stream=0):
        """Return to the training state of snapshot slot 0 or 1 (bm_net_restore)."""
        check(lib().bm_net_restore(self._n, slot, ctypes.c_void_p(stream)))

    def train_step(self, B, h, w, d_target, lr, d_grad=0, stream=0):
        loss = np.zeros(3, np.float32)
        check(lib().bm_net_train_step(self._n, B, h, w, ctypes.c_void_p(d_target), lr, ctypes.c_void_p(d_grad),
                                      loss.ctypes.data, ctypes.c_void_p(stream)))
        return loss
