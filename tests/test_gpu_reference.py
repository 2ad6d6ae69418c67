"""Engine against the reference's own kernels (compiled from the reference sources
to oracle/_ref/*.cubin and launched by oracle/refshim.c), and the oracle pinned
against the same reference runs.

Bit-exact: Lanczos up-sampling, descriptors, zero-flow initialisation (field and
the float cost D), random search (same curand XORWOW stream), the down-sampling
chain and the median.  Within 1e-4 px: the trilateral filter.  The reference's
propagation is racy (neighbours are read while other threads write them), so it
is checked through the invariants it keeps on every schedule.
"""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle
from bmtest import engine_features, engine_field, hamming_at, make_engine, random_field, random_image, set_field, small_params
from oracle import refshim

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)
if not refshim.available():
    pytest.skip("reference kernel build (oracle/_ref) not present", allow_module_level=True)

FLOW_TOL = 1e-4


@pytest.fixture(scope="module")
def ref():
    return refshim.RefKernels()


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("W,H,u", [(120, 80, 1.5), (37, 23, 2.9), (101, 67, 4.9)])
def test_upsample_matches_reference(ref, W, H, u):
    rng = np.random.default_rng(2)
    img = random_image(rng, W, H)
    prm = small_params(W, H, u, u)
    eng, _ = make_engine(prm)
    d_in = _dev(img)
    mine = torch.empty(prm.sy, prm.sx, device="cuda")
    eng.upsample(d_in.data_ptr(), mine.data_ptr())
    torch.cuda.synchronize()
    theirs = torch.empty(prm.sy, prm.sx, device="cuda")
    ref.resize_lanczos(d_in.data_ptr(), theirs.data_ptr(), W, H, prm.sx, prm.sy)
    assert torch.equal(mine, theirs)
    # the oracle's libm Lanczos against the reference's fast-math one
    assert float(np.abs(oracle.upsample(img, prm.sx, prm.sy) - theirs.cpu().numpy()).max()) <= 2e-3


@pytest.mark.parametrize("N", [32, 100, 128, 512])
def test_features_match_reference(ref, N):
    rng = np.random.default_rng(N + 1)
    prm = small_params(80, 60, 1.5, 1.5, N=N)
    eng, pattern = make_engine(prm, pattern_seed=N)
    ref.set_pattern(pattern)
    img = random_image(rng, prm.sx, prm.sy)
    d_img = _dev(img)
    ns = (N + 31) // 32
    Fr = torch.zeros(prm.sx * prm.sy * ns, dtype=torch.int32, device="cuda")
    ref.binary_features(d_img.data_ptr(), Fr.data_ptr(), prm.sx, prm.sy, N, ns)
    eng.features(d_img.data_ptr(), 1)
    torch.cuda.synchronize()
    theirs = Fr.cpu().numpy().view(np.uint32).reshape(-1, ns)
    assert np.array_equal(engine_features(eng, 1), theirs)
    # pin the oracle
    assert np.array_equal(oracle.features(img, pattern, N), theirs)


def _ref_pair(ref, prm, pattern, seed):
    from briefmatch_gb300 import synth

    f1, f2, _, _ = synth.make_pair(seed, prm.sx, prm.sy, 6.0)
    i1, i2 = f1.astype(np.float32), f2.astype(np.float32)
    ns = (prm.N + 31) // 32
    n = prm.sx * prm.sy
    bufs = {}
    for k, img in (("F1", i1), ("F2", i2)):
        d = _dev(img)
        F = torch.zeros(n * ns, dtype=torch.int32, device="cuda")
        ref.binary_features(d.data_ptr(), F.data_ptr(), prm.sx, prm.sy, prm.N, ns)
        bufs[k] = F
        bufs["img" + k] = d
    return i1, i2, bufs, ns


def test_initialize_and_random_search_match_reference(ref):
    prm = small_params(100, 70, 2.0, 2.0, N=128)
    eng, pattern = make_engine(prm)
    ref.set_pattern(pattern)
    i1, i2, b, ns = _ref_pair(ref, prm, pattern, 5)
    n = prm.sx * prm.sy
    guard = (prm.jfMax + 1) * prm.sx + prm.jfMax
    _, NX = refshim.guarded(torch, n, guard, torch.int16)
    _, NY = refshim.guarded(torch, n, guard, torch.int16)
    D = torch.zeros(n, dtype=torch.float32, device="cuda")
    state = torch.zeros(n * refshim.CURAND_STATE_BYTES, dtype=torch.uint8, device="cuda")
    ref.init_random(state.data_ptr(), prm.sx, prm.sy)
    ref.initialize(b["F1"].data_ptr(), b["F2"].data_ptr(), D.data_ptr(), NX.data_ptr(), NY.data_ptr(), prm.sx, prm.sy,
                   True, prm.N, ns)
    eng.features(b["imgF1"].data_ptr(), 0)
    eng.features(b["imgF2"].data_ptr(), 1)
    eng.initialize(True)
    nx, ny, cost, d = engine_field(eng)
    assert np.array_equal(nx, NX.cpu().numpy()) and np.array_equal(ny, NY.cpu().numpy())
    assert np.array_equal(d.view(np.uint32), D.cpu().numpy().view(np.uint32))
    dist = prm.search_dist()
    for _ in range(3):
        ref.random_search(b["F1"].data_ptr(), b["F2"].data_ptr(), D.data_ptr(), NX.data_ptr(), NY.data_ptr(),
                          state.data_ptr(), prm.sx, prm.sy, dist, prm.N, ns)
        eng.random_search()
        nx, ny, cost, d = engine_field(eng)
        assert np.array_equal(nx, NX.cpu().numpy()) and np.array_equal(ny, NY.cpu().numpy())
        assert np.array_equal(d.view(np.uint32), D.cpu().numpy().view(np.uint32))


def test_propagate_reference_invariants(ref):
    """The racy reference propagation against the engine's snapshot schedule: both
    keep D == Hamming(F1, F2 at target)/N and never increase D; the mean cost after
    the pass agrees to within the reference's own run-to-run spread plus 2%."""
    prm = small_params(110, 80, 1.5, 1.5, N=64)
    eng, pattern = make_engine(prm)
    ref.set_pattern(pattern)
    i1, i2, b, ns = _ref_pair(ref, prm, pattern, 6)
    n = prm.sx * prm.sy
    F1 = b["F1"].cpu().numpy().view(np.uint32).reshape(-1, ns)
    F2 = b["F2"].cpu().numpy().view(np.uint32).reshape(-1, ns)
    rng = np.random.default_rng(6)
    NX0, NY0 = random_field(rng, prm.sx, prm.sy, 15)
    H0 = hamming_at(F1, F2, prm.sx, NX0, NY0)
    means = []
    guard = (prm.jfMax + 1) * prm.sx + prm.jfMax
    for rep in range(3):
        _, NX = refshim.guarded(torch, n, guard, torch.int16)
        _, NY = refshim.guarded(torch, n, guard, torch.int16)
        NX.copy_(torch.from_numpy(NX0))
        NY.copy_(torch.from_numpy(NY0))
        D = torch.from_numpy((H0.astype(np.float32) / np.float32(prm.N))).cuda()
        ref.propagate(b["F1"].data_ptr(), b["F2"].data_ptr(), D.data_ptr(), NX.data_ptr(), NY.data_ptr(), prm.sx,
                      prm.sy, -1, prm.jfMax, True, prm.N, ns)
        rx, ry, rd = NX.cpu().numpy(), NY.cpu().numpy(), D.cpu().numpy()
        h = hamming_at(F1, F2, prm.sx, rx, ry)
        assert np.array_equal(np.rint(rd * prm.N).astype(np.uint16), h)
        assert (h <= H0).all()
        means.append(float(h.mean()))
    eng.features(b["imgF1"].data_ptr(), 0)
    eng.features(b["imgF2"].data_ptr(), 1)
    set_field(eng, NX0, NY0, H0)
    eng.propagate(-1)
    nx, ny, cost, _ = engine_field(eng)
    assert np.array_equal(cost, hamming_at(F1, F2, prm.sx, nx, ny)) and (cost <= H0).all()
    spread = max(means) - min(means)
    assert abs(float(cost.mean()) - np.mean(means)) <= spread + 0.02 * np.mean(means)


def test_downsample_chain_matches_reference(ref):
    W, H = 120, 80
    prm = small_params(W, H, 2.9, 2.9, N=32)
    eng, _ = make_engine(prm)
    rng = np.random.default_rng(8)
    NX, NY = random_field(rng, prm.sx, prm.sy, 20)
    set_field(eng, NX, NY, np.zeros(prm.sx * prm.sy, np.uint16))
    eng.downsample()
    torch.cuda.synchronize()
    mine = eng.read_buffer(bm.BM_BUF_FLOW_IN, np.float32).reshape(2, H, W)
    taps = prm.gauss_taps()
    ref.set_kernel(taps)
    n = prm.sx * prm.sy
    for comp, field, m in ((0, NX, np.float32(W) / np.float32(prm.sx)), (1, NY, np.float32(H) / np.float32(prm.sy))):
        src = _dev(field)
        XF = torch.zeros(n, device="cuda")
        tmp = torch.zeros(n, device="cuda")
        XI = torch.zeros(W * H, device="cuda")
        ref.convert(src.data_ptr(), XF.data_ptr(), prm.sx, prm.sy)
        ref.filter_const(XF.data_ptr(), tmp.data_ptr(), taps.size, 1, prm.sx, prm.sy)
        ref.filter_const(tmp.data_ptr(), XF.data_ptr(), taps.size, 0, prm.sx, prm.sy)
        ref.resize_nn(XF.data_ptr(), XI.data_ptr(), prm.sx, prm.sy, W, H)
        ref.mult(XI.data_ptr(), float(m), W, H)
        theirs = XI.cpu().numpy().reshape(H, W)
        assert np.array_equal(mine[comp], theirs)
        # pin the oracle (given the device's nearest-neighbour index tables)
        ou, ov = oracle.downsample(NX, NY, prm.sx, prm.sy, W, H, taps, eng.nn_indices())
        assert np.array_equal((ou, ov)[comp], theirs)


@pytest.mark.parametrize("fsize", [9, 13, 23])
def test_median_and_trilateral_match_reference(ref, fsize):
    W, H = 97, 61
    prm = small_params(W, H, 1.5, 1.5, N=32)
    prm.fsize = fsize
    eng, _ = make_engine(prm)
    rng = np.random.default_rng(fsize + 100)
    U = (rng.normal(0, 4, size=(H, W)) + np.linspace(-8, 8, W)[None, :]).astype(np.float32)
    V = rng.normal(0, 4, size=(H, W)).astype(np.float32)
    I = random_image(rng, W, H)
    eng.write_buffer(bm.BM_BUF_FLOW_IN, np.concatenate([U.ravel(), V.ravel()]))
    d_I = _dev(I)
    eng.process(d_I.data_ptr())
    torch.cuda.synchronize()
    med = eng.read_buffer(bm.BM_BUF_FLOW_MED, np.float32).reshape(2, H, W)
    out = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, H, W)
    n = W * H
    guard = (fsize // 2 + 1) * W + fsize
    meds = []
    for comp, A in ((0, U), (1, V)):
        _, src = refshim.guarded(torch, n, guard, torch.float32)
        _, tmp = refshim.guarded(torch, n, guard, torch.float32)
        dst = torch.zeros(n, device="cuda")
        src.copy_(torch.from_numpy(A.ravel()))
        ref.median(src.data_ptr(), tmp.data_ptr(), 1, fsize, W, H)
        ref.median(tmp.data_ptr(), dst.data_ptr(), 0, fsize, W, H)
        theirs = dst.cpu().numpy().reshape(H, W)
        assert np.array_equal(med[comp], theirs)
        meds.append(dst)
    dU, dV = _dev(U), _dev(V)
    Uo = torch.zeros(n, device="cuda")
    Vo = torch.zeros(n, device="cuda")
    ref.cb_filter(dU.data_ptr(), dV.data_ptr(), Uo.data_ptr(), Vo.data_ptr(), meds[0].data_ptr(), meds[1].data_ptr(),
                  d_I.data_ptr(), prm.sEPE * prm.sEPE, prm.sI * prm.sI, prm.sS * prm.sS, W, H)
    tu, tv = Uo.cpu().numpy().reshape(H, W), Vo.cpu().numpy().reshape(H, W)
    err = max(np.abs(out[0] - tu).max(), np.abs(out[1] - tv).max())
    assert err <= FLOW_TOL, err
    # pin the oracle's trilateral filter against the reference's
    _, _, ou, ov = oracle.refine(U, V, I, fsize, prm.sEPE, prm.sI, prm.sS)
    assert max(np.abs(ou - tu).max(), np.abs(ov - tv).max()) <= FLOW_TOL
