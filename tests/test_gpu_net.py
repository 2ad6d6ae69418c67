"""The proposal network's tensor-core kernels against the FP32 CPU restatement
(oracle/net_oracle.py): forward output, loss terms and every layer's gradient, on
both tensor-core paths (tcgen05 MMAs into tensor memory, the default, and mma.sync);
the two paths against each other on images wider than one 128-cell MMA tile."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import net_oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import briefmatch_gb300 as bm  # noqa: E402
from briefmatch_gb300.proposal import ProposalNet, param_count  # noqa: E402


def _bf16_bits(x):
    a = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return (((a + 0x7FFF + ((a >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def _setup(B=2, h=20, w=36, seed=0):
    rng = np.random.default_rng(seed)
    net = ProposalNet(B, h, w)
    p = net.params()
    p += rng.normal(0, 0.02, p.size).astype(np.float32)  # non-zero biases too
    net.set_params(p)
    x = rng.uniform(-1, 1, (B, h, w, net_oracle.CIN[0])).astype(np.float32)
    d_in = torch.from_numpy(_bf16_bits(x).view(np.int16)).cuda()
    net.set_input(d_in.data_ptr(), B, h, w)
    tgt = np.zeros((B, h, w, 3), np.float32)
    tgt[..., 0] = rng.normal(0, 1.5, (B, h, w))
    tgt[..., 1] = rng.normal(0, 1.5, (B, h, w))
    tgt[..., 2] = (rng.uniform(size=(B, h, w)) > 0.1).astype(np.float32)
    return net, p, x, tgt


def test_param_count():
    assert param_count() == 5 * (32 * 9 * 32 + 32) + 3 * 9 * 32 + 3


def test_input_preparation():
    """bm_net_prepare: channel 4*j + i of cell (x, y) is pixel (4x + i, 4y + j) of frame 0
    scaled to [-1, 1] (BF16), channels 16..31 the same for frame 1."""
    W, H = 40, 24
    rng = np.random.default_rng(9)
    f0 = rng.integers(0, 256, (H, W), dtype=np.uint8)
    f1 = rng.integers(0, 256, (H, W), dtype=np.uint8)
    h4, w4 = H // 4, W // 4
    net = ProposalNet(1, h4, w4)
    p = net.params()
    p[:] = 0
    # layers 0-4: identity on all 32 channels through the centre tap (ReLU keeps the
    # non-negative inputs); the head reads frame-0 pixel (0, 0) as u and frame-1
    # pixel (3, 3) as v
    d0, d1 = torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda()
    net.prepare(0, d0.data_ptr(), d1.data_ptr(), W, H)
    k = 0
    dims = list(zip(net_oracle.CIN, net_oracle.COUT))
    for l, (ci, co) in enumerate(dims):
        Wl = np.zeros((co, 9, ci), np.float32)
        if l < 5:
            for c in range(min(ci, co)):
                Wl[c, 4, c] = 1.0
        else:
            Wl[0, 4, 0] = 1.0
            Wl[1, 4, 16 + 15] = 1.0
        p[k:k + co * 9 * ci] = Wl.ravel()
        k += co * 9 * ci + co
    net.set_params(p)
    out = torch.empty(1, h4, w4, 3, device="cuda")
    net.forward(1, h4, w4, out.data_ptr())
    torch.cuda.synchronize()
    o = out[0].cpu().numpy()
    bf = lambda a: net_oracle.bf16(a.astype(np.float32) / np.float32(127.5) - np.float32(1.0))
    want_u = np.maximum(bf(f0[0::4, 0::4]), 0)
    want_v = np.maximum(bf(f1[3::4, 3::4]), 0)
    assert np.array_equal(o[..., 0], want_u) and np.array_equal(o[..., 1], want_v)


@pytest.mark.parametrize("reduce,W,H", [(1, 40, 24), (2, 70, 45), (4, 70, 45)])
def test_input_preparation_reduced(reduce, W, H):
    """bm_net_prepare_reduced against net_oracle.net_input, every channel and sign: a
    probe network passes input channel c of both frames through the centre taps as
    relu(x) - relu(-x) = x, so the head outputs the BF16 input values exactly."""
    rng = np.random.default_rng(10 + reduce)
    f0 = rng.integers(0, 256, (H, W), dtype=np.uint8)
    f1 = rng.integers(0, 256, (H, W), dtype=np.uint8)
    want = net_oracle.bf16(net_oracle.net_input(f0, f1, reduce))
    h4, w4 = H // reduce // 4, W // reduce // 4
    assert want.shape == (h4, w4, 32)
    net = ProposalNet(1, H // 4, W // 4)
    d0, d1 = torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda()
    net.prepare(0, d0.data_ptr(), d1.data_ptr(), W, H, reduce=reduce)
    out = torch.empty(1, h4, w4, 3, device="cuda")
    dims = list(zip(net_oracle.CIN, net_oracle.COUT))
    for c in range(16):
        p = np.zeros(param_count(), np.float32)
        k = 0
        for l, (ci, co) in enumerate(dims):
            Wl = np.zeros((co, 9, ci), np.float32)
            if l == 0:
                Wl[0, 4, c], Wl[1, 4, c], Wl[2, 4, 16 + c], Wl[3, 4, 16 + c] = 1, -1, 1, -1
            elif l < 5:
                for q in range(4):
                    Wl[q, 4, q] = 1
            else:
                Wl[0, 4, 0], Wl[0, 4, 1], Wl[1, 4, 2], Wl[1, 4, 3] = 1, -1, 1, -1
            p[k:k + co * 9 * ci] = Wl.ravel()
            k += co * 9 * ci + co
        net.set_params(p)
        net.forward(1, h4, w4, out.data_ptr())
        torch.cuda.synchronize()
        o = out[0].cpu().numpy()
        assert np.array_equal(o[..., 0], want[..., c]), (reduce, c)
        assert np.array_equal(o[..., 1], want[..., 16 + c]), (reduce, c)
    net.close()


def test_input_reduction_rejected():
    net = ProposalNet(1, 8, 8)
    d = torch.zeros(32, 32, dtype=torch.uint8, device="cuda")
    with pytest.raises(bm.BriefMatchException, match="reduce must be 1, 2 or 4"):
        net.prepare(0, d.data_ptr(), d.data_ptr(), 32, 32, reduce=3)
    with pytest.raises(bm.BriefMatchException, match="beyond the network's buffers"):
        net.prepare(0, d.data_ptr(), d.data_ptr(), 12, 32, reduce=4)  # (12 / 4) / 4 = 0 cells
    net.close()


def test_snapshot_restore_returns_to_the_training_state():
    """bm_net_snapshot / bm_net_restore: after Adam steps, restoring slot 0 gives back
    the parameters and the forward output of the snapshot, and the Adam moments too
    (the same steps from there reach the same parameters); slot 1 keeps its own state;
    a slot never written is refused."""
    B, h, w = 2, 12, 20
    net, p0, x, tgt = _setup(B, h, w, seed=5)
    d_t = torch.from_numpy(tgt).cuda()
    out = torch.empty(B, h, w, 3, device="cuda")

    def fwd():
        net.forward(B, h, w, out.data_ptr())
        torch.cuda.synchronize()
        return out.cpu().numpy().copy()

    def steps(k):
        for _ in range(k):
            net.train_step(B, h, w, d_t.data_ptr(), 1e-2)
        torch.cuda.synchronize()

    with pytest.raises(bm.BriefMatchException, match="no snapshot"):
        net.restore(0)
    with pytest.raises(bm.BriefMatchException, match="slot not 0 or 1"):
        net.snapshot(2)
    steps(2)
    net.snapshot(0)
    torch.cuda.synchronize()
    pa, oa = net.params(), fwd()
    steps(3)
    pb = net.params()
    assert not np.array_equal(pa, pb)
    net.snapshot(1)
    net.restore(0)
    torch.cuda.synchronize()
    assert np.array_equal(net.params(), pa) and np.array_equal(fwd(), oa)
    steps(3)
    # FP32 atomics in the weight gradients may sum in another order, which can flip
    # the sign of Adam's step for a parameter whose gradient is near zero: all but a
    # handful of parameters replay the same steps
    pr = net.params()
    assert np.mean(np.abs(pr - pb) > 1e-5) < 1e-3, np.sort(np.abs(pr - pb))[-5:]
    assert np.mean(np.abs(pr - pb)) < 1e-3 * np.mean(np.abs(pb - pa))
    net.restore(1)
    torch.cuda.synchronize()
    assert np.array_equal(net.params(), pb)
    net.close()


def test_tcgen05_path_is_the_default():
    net = ProposalNet(1, 8, 8)
    assert net.umma == 1
    assert net.fused_ctas >= 152  # the fused launch is available as mode 2
    net.close()


@pytest.mark.parametrize("umma", [2, 1, 0])
def test_forward_matches_oracle(umma):
    B, h, w = 2, 20, 36
    net, p, x, _ = _setup(B, h, w)
    net.set_umma(umma)
    out = torch.empty(B, h, w, 3, device="cuda")
    net.forward(B, h, w, out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    net.check()
    want, _ = net_oracle.forward(p, x)
    err = np.abs(got - want).max() / max(1e-6, np.abs(want).max())
    assert err < 2e-2, err


@pytest.mark.parametrize("umma", [2, 1, 0])
def test_gradients_match_oracle(umma):
    B, h, w = 2, 20, 36
    net, p, x, tgt = _setup(B, h, w, seed=1)
    net.set_umma(umma)
    d_t = torch.from_numpy(tgt).cuda()
    d_g = torch.empty(param_count(), device="cuda")
    loss = net.train_step(B, h, w, d_t.data_ptr(), 0.0, d_g.data_ptr())
    torch.cuda.synchronize()
    got = d_g.cpu().numpy()
    out, acts = net_oracle.forward(p, x)
    dY, losses = net_oracle.loss_grad(out, tgt)
    want = net_oracle.backward(p, x, acts, dY)
    assert np.allclose(loss, losses, rtol=2e-2, atol=1e-5), (loss, losses)
    k = 0
    for l, (ci, co) in enumerate(zip(net_oracle.CIN, net_oracle.COUT)):
        n = co * 9 * ci + co
        g, wv = got[k:k + n], want[k:k + n]
        rel = np.linalg.norm(g - wv) / max(1e-12, np.linalg.norm(wv))
        assert rel < 3e-2, (l, rel)
        k += n


def test_training_reduces_loss():
    B, h, w = 4, 24, 32
    net, p, x, tgt = _setup(B, h, w, seed=2)
    d_t = torch.from_numpy(tgt).cuda()
    first = net.train_step(B, h, w, d_t.data_ptr(), 1e-3)
    for _ in range(60):
        last = net.train_step(B, h, w, d_t.data_ptr(), 1e-3)
    assert last[0] < 0.8 * first[0]


@pytest.mark.parametrize("B,h,w", [(1, 109, 256), (2, 7, 300), (3, 5, 17), (1, 300, 480)])
@pytest.mark.parametrize("mode", [2, 1])
def test_tcgen05_equals_mma_sync(mode, B, h, w):
    """Whole 128-cell tiles, a ragged last tile, an image narrower than one tile and
    one with more tiles than co-resident CTAs (each CTA of the fused launch then walks
    several tiles per layer): the tcgen05 forward and training step equal the
    mma.sync ones up to FP32 summation order (both round activations to BF16 between
    layers)."""
    net, p, x, tgt = _setup(B, h, w, seed=3)
    d_t = torch.from_numpy(tgt).cuda()
    outs, grads = [], []
    for umma in (mode, 0):
        net.set_umma(umma)
        out = torch.empty(B, h, w, 3, device="cuda")
        net.forward(B, h, w, out.data_ptr())
        g = torch.empty(param_count(), device="cuda")
        net.train_step(B, h, w, d_t.data_ptr(), 0.0, g.data_ptr())
        torch.cuda.synchronize()
        net.check()
        outs.append(out.cpu().numpy())
        grads.append(g.cpu().numpy())
    scale = max(1e-6, float(np.abs(outs[1]).max()))
    assert float(np.abs(outs[0] - outs[1]).max()) / scale < 1e-2
    rel = np.linalg.norm(grads[0] - grads[1]) / max(1e-12, np.linalg.norm(grads[1]))
    assert rel < 2e-2, rel
    net.close()
