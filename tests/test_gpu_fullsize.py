"""The engine at the workload's full sizes -- 1024x436 u2.9 N128 (3.75 Mpx up-sampled)
and 1920x1080 u4.9 N512 (49.8 Mpx up-sampled, 3.2 GB of descriptors per frame) --
checked against the oracle where the oracle can follow in seconds and by
size-independent properties elsewhere:

- descriptors of a band of rows bit-exact vs the oracle run on a crop of the
  engine's up-sampled image that holds every row the band's samples reach;
- the matched field: every stored cost equals the Hamming distance at the stored
  vector, every vector keeps its target inside the image, and matching lowers the
  mean cost far below the zero field's;
- the down-sampled flow bit-exact vs the oracle over the whole frame;
- the refined flow on a band of rows (crop with the filters' full reach): the
  median bit-exact vs the oracle; the trilateral output within 1e-4 px of a float64
  evaluation of the filter, and of the oracle within 1e-4 px at 2304 taps per pixel
  and 3e-4 px at 8836.  The oracle follows the reference's order -- one float sum
  over all taps -- whose own rounding reaches ~1.1e-4 px at 8836 taps (sums of
  ~1200 weights times flows of ~12 px); the engine's column-wise sums stay within
  ~5e-6 px of float64 there.
"""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle
from bmtest import trilateral_f64

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

from briefmatch_gb300 import synth  # noqa: E402

FLOW_TOL = 1e-4
CONFIGS = [(1024, 436, 2.9, 128, 15.0), (1920, 1080, 4.9, 512, 24.0)]

_LUT = torch.tensor([bin(i).count("1") for i in range(256)], dtype=torch.int32)


def _popcount_rows(x):
    """Bit count of each row of an int32 CUDA tensor [n][w]."""
    lut = _LUT.to(x.device)
    return lut[x.contiguous().view(torch.uint8).long()].view(x.shape[0], -1).sum(dim=1)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _read_dev(eng, which, dst):
    """Device copy of a context buffer into a CUDA tensor, complete on return (the
    context's stream is its own, not torch's)."""
    nbytes = dst.numel() * dst.element_size()
    bm.check(bm.lib().bm_read_buffer(eng.ctx, which, bm.ctypes.c_void_p(dst.data_ptr()), nbytes, 1))
    eng.synchronize()
    return dst


@pytest.mark.parametrize("W,H,u,N,vmax", CONFIGS, ids=["1024x436_u2.9_N128", "1920x1080_u4.9_N512"])
def test_full_size_pair(W, H, u, N, vmax):
    prm = bm.BMParams.derive(W, H, u, u, N=N)
    eng = bm.BriefMatch(prm)
    eng.setup()
    pattern = prm.make_pattern(11)
    eng.set_pattern(pattern)
    sx, sy, n = prm.sx, prm.sy, prm.sx * prm.sy
    f0, f1, _, _ = synth.make_pair(77, W, H, vmax)
    d0, d1 = _dev(f0), _dev(f1)
    up0 = torch.empty(sy, sx, device="cuda")
    up1 = torch.empty(sy, sx, device="cuda")
    torch.cuda.synchronize()   # the frames' uploads, before the context's own stream reads them
    eng.upsample_u8(d0.data_ptr(), up0.data_ptr())
    eng.upsample_u8(d1.data_ptr(), up1.data_ptr())
    eng.features(up0.data_ptr(), 0)
    eng.synchronize()

    # descriptors of a band of rows vs the oracle on a crop holding their reach
    nsp = eng.feature_stride()
    ns = (N + 31) // 32
    reach = int(np.abs(np.trunc(pattern.reshape(-1, 4)[:, [1, 3]])).max()) + 1
    y0, rows = sy // 2, 3
    c0, c1 = max(0, y0 - reach), min(sy, y0 + rows + reach)
    crop = up0[c0:c1].cpu().numpy()
    F_or = oracle.features(crop, pattern, N).reshape(c1 - c0, sx, ns)[y0 - c0:y0 - c0 + rows]
    F1 = _read_dev(eng, bm.BM_BUF_FEAT1, torch.empty(n * nsp, dtype=torch.int32, device="cuda"))
    band = F1.view(sy, sx, nsp)[y0:y0 + rows, :, :ns].cpu().numpy().view(np.uint32)
    assert np.array_equal(band, F_or)
    assert not F1.view(n, nsp)[:, ns:].any().item(), "descriptor padding words must be zero"

    # match: the field's invariants over every pixel
    eng.match(up0.data_ptr(), up1.data_ptr())
    eng.synchronize()
    F2 = _read_dev(eng, bm.BM_BUF_FEAT2, torch.empty_like(F1))
    field = _read_dev(eng, bm.BM_BUF_FLOW, torch.empty(n, dtype=torch.int32, device="cuda"))
    cost = _read_dev(eng, bm.BM_BUF_COST, torch.empty(n, dtype=torch.int16, device="cuda"))
    nx = (field & 0xFFFF).to(torch.int16).long()
    ny = (field >> 16).to(torch.int16).long()
    pix = torch.arange(n, device="cuda", dtype=torch.int64)
    xs, ys = pix % sx, pix // sx
    assert bool(((xs + nx >= 0) & (xs + nx < sx) & (ys + ny >= 0) & (ys + ny < sy)).all())
    A = F1.view(n, nsp)[:, :ns]
    B = F2.view(n, nsp)[:, :ns]
    chunk = 1 << 21
    zero_sum = 0
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        q = pix[s:e] + nx[s:e] + ny[s:e] * sx
        h = _popcount_rows(A[s:e] ^ B[q])
        assert torch.equal(h.to(torch.int32), cost[s:e].to(torch.int32) & 0xFFFF), "cost != Hamming at stored vector"
        zero_sum += int(_popcount_rows(A[s:e] ^ B[s:e]).sum().item())
    mean_cost = float((cost.to(torch.int32) & 0xFFFF).double().mean().item())
    assert mean_cost < 0.5 * zero_sum / n, (mean_cost, zero_sum / n)

    # down-sampling over the whole frame, bit-exact
    eng.downsample()
    eng.synchronize()
    NX = nx.to(torch.int16).cpu().numpy()
    NY = ny.to(torch.int16).cpu().numpy()
    U, V = oracle.downsample(NX, NY, sx, sy, W, H, prm.gauss_taps(), eng.nn_indices())
    uv_in = eng.read_buffer(bm.BM_BUF_FLOW_IN, np.float32).reshape(2, H, W)
    assert np.array_equal(uv_in[0], U) and np.array_equal(uv_in[1], V)

    # refinement of a band of rows vs the oracle on a crop with the filters' reach
    guide = d0.float()
    torch.cuda.synchronize()
    eng.process(guide.data_ptr())
    eng.synchronize()
    out = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, H, W)
    s = int(np.ceil(2.5 * prm.sS))
    margin = s + prm.fsize
    r0, rr = H // 2, 4
    a, b = r0 - margin, r0 + rr + margin
    Um, Vm, Uo, Vo = oracle.refine(U[a:b], V[a:b], f0[a:b].astype(np.float32), prm.fsize, prm.sEPE, prm.sI, prm.sS)
    med = eng.read_buffer(bm.BM_BUF_FLOW_MED, np.float32).reshape(2, H, W)
    assert np.array_equal(med[0, r0:r0 + rr], Um[margin:margin + rr])
    assert np.array_equal(med[1, r0:r0 + rr], Vm[margin:margin + rr])
    err = max(np.abs(out[0, r0:r0 + rr] - Uo[margin:margin + rr]).max(),
              np.abs(out[1, r0:r0 + rr] - Vo[margin:margin + rr]).max())
    assert err <= (FLOW_TOL if s <= 24 else 3 * FLOW_TOL), err
    ex_u, ex_v = trilateral_f64(U, V, med[0], med[1], f0, r0, rr, s, prm.sEPE, prm.sI, prm.sS)
    err64 = max(np.abs(out[0, r0:r0 + rr] - ex_u).max(), np.abs(out[1, r0:r0 + rr] - ex_v).max())
    assert err64 <= FLOW_TOL, err64
    eng.clean()
