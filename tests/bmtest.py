"""Shared helpers for the parity tests (engine through its C ABI vs the oracle)."""
from __future__ import annotations

import numpy as np

import briefmatch_gb300 as bm


def small_params(W=120, H=80, ux=1.5, uy=1.5, N=64, **kw):
    return bm.BMParams.derive(W, H, ux, uy, N=N, **kw)


def make_engine(prm, pattern_seed=3):
    import torch

    eng = bm.BriefMatch(prm)
    eng.setup()
    pattern = prm.make_pattern(pattern_seed)
    eng.set_pattern(pattern)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    return eng, pattern


def engine_features(eng, slot):
    """Engine descriptors of a slot in the reference layout [npix][ceil(N/32)],
    plus a check that the padding words are zero."""
    p = eng.params
    nsp = eng.feature_stride()
    ns = (p.N + 31) // 32
    which = bm.BM_BUF_FEAT1 if slot == 0 else bm.BM_BUF_FEAT2
    F = eng.read_buffer(which, np.uint32, p.sx * p.sy * nsp).reshape(-1, nsp)
    assert not F[:, ns:].any(), "descriptor padding words must be zero"
    return np.ascontiguousarray(F[:, :ns])


def engine_field(eng):
    """(NX, NY, cost, D) of the engine's current field."""
    import torch

    p = eng.params
    n = p.sx * p.sy
    nx = torch.empty(n, dtype=torch.int16, device="cuda")
    ny = torch.empty(n, dtype=torch.int16, device="cuda")
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    eng.export_field(nx.data_ptr(), ny.data_ptr(), d.data_ptr())
    torch.cuda.synchronize()
    cost = eng.read_buffer(bm.BM_BUF_COST, np.uint16, n)
    return nx.cpu().numpy(), ny.cpu().numpy(), cost, d.cpu().numpy()


def set_field(eng, NX, NY, cost):
    import torch

    tx = torch.from_numpy(np.ascontiguousarray(NX, np.int16)).cuda()
    ty = torch.from_numpy(np.ascontiguousarray(NY, np.int16)).cuda()
    tc = torch.from_numpy(np.ascontiguousarray(cost, np.uint16).view(np.int16)).cuda()
    eng.import_field(tx.data_ptr(), ty.data_ptr(), tc.data_ptr())
    torch.cuda.synchronize()


def engine_normals(eng, call):
    import torch

    p = eng.params
    out = torch.empty(p.sx * p.sy * 2, dtype=torch.float32, device="cuda")
    eng.normals(call, out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def random_image(rng, w, h):
    """Smooth random image in [0,255] (so descriptors are not dominated by ties)."""
    from briefmatch_gb300 import synth

    return synth.make_frame(rng, w, h, blobs=12).astype(np.float32)


def random_field(rng, sx, sy, vmax):
    """A valid field: each vector keeps its target inside the image."""
    ys, xs = np.mgrid[0:sy, 0:sx]
    nx = rng.integers(-vmax, vmax + 1, size=(sy, sx))
    ny = rng.integers(-vmax, vmax + 1, size=(sy, sx))
    nx = np.clip(nx, -xs, sx - xs - 1).astype(np.int16).ravel()
    ny = np.clip(ny, -ys, sy - ys - 1).astype(np.int16).ravel()
    return nx, ny


def hamming_at(F1, F2, sx, NX, NY):
    """Hamming distance of every pixel's descriptor to the target of its vector."""
    n = F1.shape[0]
    p = np.arange(n)
    q = p + NX.astype(np.int64) + NY.astype(np.int64) * sx
    x = F1 ^ F2[q]
    return np.unpackbits(x.view(np.uint8), axis=1).sum(axis=1).astype(np.uint16)


def trilateral_f64(U, V, Um, Vm, I, r0, rows, s, sEPE, sI, sS):
    """The cross-trilateral filter (briefmatch_cuda.cu:248-297: clamp-to-edge window
    [-s, s)^2, weights exp(-EPE^2/2sEPE^2) exp(-dI^2/2sI^2) exp(-d^2/2sS^2) with
    intensities / 255, weight sum floored at 1e-5) in float64, rows r0..r0+rows."""
    H, W = U.shape
    js, is_ = np.mgrid[-s:s, -s:s]
    sp = (is_ ** 2 + js ** 2) / (2.0 * sS * sS)
    outu = np.empty((rows, W))
    outv = np.empty((rows, W))
    for r in range(rows):
        y = r0 + r
        ys = np.clip(y + js, 0, H - 1)
        for x0 in range(0, W, 128):
            xs_c = np.arange(x0, min(W, x0 + 128))
            xs = np.clip(xs_c[:, None, None] + is_[None], 0, W - 1)
            yy = np.broadcast_to(ys[None], xs.shape)
            u1 = U[yy, xs].astype(np.float64)
            v1 = V[yy, xs].astype(np.float64)
            du = u1 - Um[y, xs_c][:, None, None]
            dv = v1 - Vm[y, xs_c][:, None, None]
            dI = (I[yy, xs].astype(np.float64) - I[y, xs_c].astype(np.float64)[:, None, None]) / 255.0
            w = np.exp(-(du * du + dv * dv) / (2.0 * sEPE * sEPE) - dI * dI / (2.0 * sI * sI) - sp[None])
            Wt = np.maximum(w.sum(axis=(1, 2)), 1e-5)
            outu[r, xs_c] = (w * u1).sum(axis=(1, 2)) / Wt
            outv[r, xs_c] = (w * v1).sum(axis=(1, 2)) / Wt
    return outu, outv
