"""Colour coding on the GPU (bm_colors: BriefMatch::computeColors, briefmatch.cpp:373-421,
with util/colorcode.cpp:52-74; bm_flow_colors for any device field) against the
oracle's restatement, byte for byte: every wheel segment, vectors inside and outside
the unit disc, unknown vectors (NaN, |v| > 1e9), zero vectors, a fixed and a measured
motion range."""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

from briefmatch_gb300 import synth  # noqa: E402


def _field(seed, h, w, scale):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(-np.pi, np.pi, size=(h, w))
    mag = rng.uniform(0, 1.6, size=(h, w)) * scale
    U = (mag * np.cos(ang)).astype(np.float32)
    V = (mag * np.sin(ang)).astype(np.float32)
    U[0, :6] = [0, np.nan, 2e9, -3e9, 0, 1e-30]
    V[0, :6] = [0, 0, 0, 1, np.inf, 0]
    # exact multiples of the wheel's angular step and the unit radius
    k = np.arange(w)
    U[1] = (scale * np.cos(2 * np.pi * k / 54)).astype(np.float32)
    V[1] = (scale * np.sin(2 * np.pi * k / 54)).astype(np.float32)
    return U, V


@pytest.mark.parametrize("max_motion", [4.0, 1.0, 37.5])
def test_flow_colors_match_oracle(max_motion):
    U, V = _field(1, 300, 400, 4.0)
    dU, dV = torch.from_numpy(U).cuda(), torch.from_numpy(V).cuda()
    out = torch.zeros(300, 400, 3, dtype=torch.uint8, device="cuda")
    bm.flow_colors(dU.data_ptr(), dV.data_ptr(), 400, 300, max_motion, out.data_ptr(),
                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = oracle.flow_colors(U, V, max_motion)
    assert np.array_equal(got, want), int((got != want).sum())
    assert (got[0, 1] == 0).all() and (got[0, 2] == 0).all()  # unknown -> black
    assert np.unique(got.reshape(-1, 3), axis=0).shape[0] > 5000


def test_flow_colors_rejects_bad_range():
    d = torch.zeros(4, device="cuda")
    o = torch.zeros(12, dtype=torch.uint8, device="cuda")
    for mm in (0.0, -1.0, float("nan"), float("inf")):
        with pytest.raises(bm.BriefMatchException):
            bm.flow_colors(d.data_ptr(), d.data_ptr(), 2, 2, mm, o.data_ptr())


@pytest.mark.parametrize("maxmot", [0.0, 3.0])
def test_context_colors_match_oracle(maxmot):
    """The context's output field (what bm_convert returns) coloured by bm_colors, to
    host and to device memory."""
    W, H = 160, 96
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64, maxmot=maxmot)
    eng = bm.FlowEngine(prm)
    f1, f2, _, _ = synth.make_pair(12, W, H, 6.0)
    eng.process_frame(f1)
    eng.process_frame(f2)
    u, v = eng.convert()
    host = eng.compute_colors()
    dev = torch.zeros(H, W, 3, dtype=torch.uint8, device="cuda")
    eng.compute_colors(dev.data_ptr())
    eng.synchronize()
    want = oracle.flow_colors(u, v, maxmot)
    assert np.array_equal(host, want)
    assert np.array_equal(dev.cpu().numpy(), want)
    eng.clean()


def test_context_colors_of_an_all_zero_field():
    """No motion at all: the measured range is 0 and counts as 1 (briefmatch.cpp:405)."""
    W, H = 64, 48
    prm = bm.BMParams.derive(W, H, 1.0, 1.0, N=32, maxmot=0.0)
    eng = bm.FlowEngine(prm)
    f = synth.make_pair(3, W, H, 0.0)[0]
    eng.process_frame(f)
    eng.process_frame(f)
    u, v = eng.convert()
    assert not u.any() and not v.any()
    assert np.array_equal(eng.compute_colors(), oracle.flow_colors(u, v, 0.0))
    eng.clean()
