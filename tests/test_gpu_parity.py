"""Engine (through its C ABI) against the oracle, stage by stage and end to end.

Bar: descriptors, Hamming costs, the field and the down-sampled and median-filtered
flow bit-exact; the refined flow within 1e-4 px max-abs; the Lanczos up-sampling
(sin and division are fast-math intrinsics on the GPU, libm in the oracle) within
the tolerance stated in the test.
"""
from __future__ import annotations

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle
from bmtest import (engine_features, engine_field, engine_normals, hamming_at, make_engine, random_field,
                    random_image, set_field, small_params)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

FLOW_TOL = 1e-4      # refined flow, px max-abs
UPSAMPLE_TOL = 2e-3  # up-sampled intensity (0..255), max-abs


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _upsampled(eng, img):
    p = eng.params
    d_in = _dev(img.astype(np.float32))
    d_up = torch.empty(p.sy, p.sx, dtype=torch.float32, device="cuda")
    eng.upsample(d_in.data_ptr(), d_up.data_ptr())
    torch.cuda.synchronize()
    return d_up


@pytest.mark.parametrize("W,H,u", [(120, 80, 1.5), (37, 23, 2.9), (64, 48, 1.0), (101, 67, 4.9)])
def test_upsample_vs_oracle(W, H, u):
    rng = np.random.default_rng(1)
    img = random_image(rng, W, H)
    prm = small_params(W, H, u, u)
    eng, _ = make_engine(prm)
    d_up = _upsampled(eng, img)
    ref = oracle.upsample(img, prm.sx, prm.sy)
    diff = np.abs(d_up.cpu().numpy() - ref).max()
    assert diff <= UPSAMPLE_TOL, diff
    # the 8-bit entry point computes the same values
    u8 = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    d8 = _dev(u8)
    out8 = torch.empty(prm.sy, prm.sx, device="cuda")
    eng.upsample_u8(d8.data_ptr(), out8.data_ptr())
    d_upf = _upsampled(eng, u8.astype(np.float32))
    torch.cuda.synchronize()
    assert torch.equal(out8, d_upf)


@pytest.mark.parametrize("N", [2, 31, 32, 64, 96, 128, 200, 512])
def test_features_bit_exact(N):
    rng = np.random.default_rng(N)
    prm = small_params(90, 60, 1.5, 1.5, N=N)
    eng, pattern = make_engine(prm, pattern_seed=N)
    img = random_image(rng, prm.sx, prm.sy)
    d_img = _dev(img)
    eng.features(d_img.data_ptr(), 1)
    torch.cuda.synchronize()
    got = engine_features(eng, 1)
    want = oracle.features(img, pattern, N)
    assert np.array_equal(got, want)


def test_features_border_and_interior_paths():
    # a wide pattern makes most blocks take the clamped path, a narrow one the interior path
    rng = np.random.default_rng(5)
    for area in (2.0, 40.0, 300.0):
        prm = small_params(160, 120, 1.0, 1.0, N=128)
        prm.patchArea = area
        eng, _ = make_engine(prm)
        pattern = prm.make_pattern(11)
        eng.set_pattern(pattern)
        img = random_image(rng, prm.sx, prm.sy)
        d_img = _dev(img)
        eng.features(d_img.data_ptr(), 0)
        torch.cuda.synchronize()
        assert np.array_equal(engine_features(eng, 0), oracle.features(img, pattern, 128))


@pytest.mark.parametrize("W,H,u,N", [(90, 60, 2.9, 128), (37, 23, 4.9, 64), (70, 45, 1.5, 512)])
def test_frame_features_edge_replicated(W, H, u, N):
    """bm_frame up-samples into an image with an edge-replicated margin and computes
    the descriptors there with no clamping; they must equal the oracle's clamped
    descriptors of the same up-sampled image, for the default pattern, wider ones
    (which re-allocate the margin) and a narrower one.  BM_BUF_UP gives the dense up-sampled image, equal to
    bm_upsample_u8's."""
    rng = np.random.default_rng(W)
    prm = small_params(W, H, u, u, N=N)
    eng, pattern = make_engine(prm)
    for k, area in enumerate((None, 4.0 * prm.patchArea, 16.0 * prm.patchArea, 0.25 * prm.patchArea)):
        if area is not None:
            q = small_params(W, H, u, u, N=N)
            q.patchArea = area
            pattern = q.make_pattern(20 + k)
            eng.set_pattern(pattern)
            eng.reset_sequence()
        for _ in range(2):
            u8 = np.clip(np.rint(random_image(rng, W, H)), 0, 255).astype(np.uint8)
            d8 = _dev(u8)
            eng.frame(d8.data_ptr(), True)
            ref = torch.empty(prm.sy, prm.sx, device="cuda")
            eng.upsample_u8(d8.data_ptr(), ref.data_ptr())
            eng.synchronize()
            up = eng.read_buffer(bm.BM_BUF_UP, np.float32, prm.sx * prm.sy).reshape(prm.sy, prm.sx)
            assert np.array_equal(up, ref.cpu().numpy()), (k, area)
            # the frame's descriptors are FEAT1 once bm_frame has swapped the slots
            assert np.array_equal(engine_features(eng, 0), oracle.features(up, pattern, N)), (k, area)


def _two_frames(eng, prm, pattern, seed=0):
    rng = np.random.default_rng(seed)
    f1, f2, _, _ = __import__("briefmatch_gb300.synth", fromlist=["make_pair"]).make_pair(seed, prm.sx, prm.sy, 6.0)
    i1, i2 = f1.astype(np.float32), f2.astype(np.float32)
    d1, d2 = _dev(i1), _dev(i2)
    eng.features(d1.data_ptr(), 0)
    eng.features(d2.data_ptr(), 1)
    torch.cuda.synchronize()
    F1 = oracle.features(i1, pattern, prm.N)
    F2 = oracle.features(i2, pattern, prm.N)
    assert np.array_equal(engine_features(eng, 0), F1)
    assert np.array_equal(engine_features(eng, 1), F2)
    return F1, F2, rng


def test_initialize_first():
    prm = small_params(100, 70, 1.5, 1.5, N=128)
    eng, pattern = make_engine(prm)
    F1, F2, _ = _two_frames(eng, prm, pattern)
    eng.initialize(True)
    nx, ny, cost, d = engine_field(eng)
    NX, NY, H = oracle.initialize(F1, F2, prm.sx, prm.sy, prm.N, True)
    assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)
    assert np.array_equal(np.rint(d * prm.N).astype(np.uint16), H)


def test_initialize_temporal():
    prm = small_params(100, 70, 1.5, 1.5, N=64)
    eng, pattern = make_engine(prm)
    F1, F2, rng = _two_frames(eng, prm, pattern, seed=2)
    NX0, NY0 = random_field(rng, prm.sx, prm.sy, 9)
    set_field(eng, NX0, NY0, np.zeros(prm.sx * prm.sy, np.uint16))
    eng.initialize(False)
    nx, ny, cost, _ = engine_field(eng)
    NX, NY, H = oracle.initialize(F1, F2, prm.sx, prm.sy, prm.N, False, NX0, NY0)
    assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)


@pytest.mark.parametrize("pd,double_prop,jf", [(-1, 1, 256), (1, 1, 256), (-1, 0, 64), (1, 1, 100), (-1, 1, 3)])
def test_propagate_bit_exact(pd, double_prop, jf):
    prm = small_params(110, 75, 1.5, 1.5, N=64, jfMax=jf, doubleProp=double_prop)
    eng, pattern = make_engine(prm)
    F1, F2, rng = _two_frames(eng, prm, pattern, seed=3)
    NX0, NY0 = random_field(rng, prm.sx, prm.sy, 12)
    H0 = hamming_at(F1, F2, prm.sx, NX0, NY0)
    set_field(eng, NX0, NY0, H0)
    eng.propagate(pd)
    nx, ny, cost, _ = engine_field(eng)
    NX, NY, H = oracle.propagate(F1, F2, prm.sx, prm.sy, prm.N, pd, jf, double_prop, NX0, NY0, H0)
    assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)
    assert np.array_equal(cost, hamming_at(F1, F2, prm.sx, nx, ny))
    assert (cost <= H0).all()


@pytest.mark.parametrize("rng_mode", [bm.BM_RNG_XORWOW, bm.BM_RNG_PHILOX])
def test_random_search_bit_exact(rng_mode):
    prm = small_params(100, 70, 2.0, 2.0, N=128, rng=rng_mode, seed=1234)
    eng, pattern = make_engine(prm)
    F1, F2, rng = _two_frames(eng, prm, pattern, seed=4)
    eng.initialize(True)
    NX, NY, H = oracle.initialize(F1, F2, prm.sx, prm.sy, prm.N, True)
    dist = prm.search_dist()
    for call in range(3):
        nrm = engine_normals(eng, call)
        assert np.isfinite(nrm).all() and abs(float(nrm.mean())) < 0.05 and 0.9 < float(nrm.std()) < 1.1
        eng.random_search()
        NX, NY, H = oracle.random_search(F1, F2, prm.sx, prm.sy, prm.N, dist, nrm, NX, NY, H)
        nx, ny, cost, _ = engine_field(eng)
        assert np.array_equal(nx, NX) and np.array_equal(ny, NY) and np.array_equal(cost, H)
    assert eng.rng_position() == 3


@pytest.mark.parametrize("W,H,u", [(120, 80, 2.9), (90, 64, 1.5), (64, 40, 1.0), (75, 41, 4.9)])
def test_downsample_bit_exact(W, H, u):
    prm = small_params(W, H, u, u, N=32)
    eng, _ = make_engine(prm)
    rng = np.random.default_rng(7)
    NX, NY = random_field(rng, prm.sx, prm.sy, 20)
    set_field(eng, NX, NY, np.zeros(prm.sx * prm.sy, np.uint16))
    eng.downsample()
    torch.cuda.synchronize()
    uv = eng.read_buffer(bm.BM_BUF_FLOW_IN, np.float32).reshape(2, H, W)
    taps = prm.gauss_taps()
    assert np.array_equal(taps, oracle.gauss_taps(prm.sigma))
    nn = eng.nn_indices()
    U, V = oracle.downsample(NX, NY, prm.sx, prm.sy, W, H, taps, nn)
    assert np.array_equal(uv[0], U) and np.array_equal(uv[1], V)
    # the device's tables differ from IEEE rounding by at most one pixel (half-integer quotients)
    ieee = np.floor(np.arange(W) * np.float32(prm.sx) / np.float32(W) + 0.5)
    assert np.abs(nn[0].astype(np.int64) - ieee).max() <= 1


@pytest.mark.parametrize("fsize", [1, 2, 3, 9, 12, 13, 15, 23, 30, 31, 46, 47])
def test_median_and_trilateral(fsize):
    W, H = 97, 61
    prm = small_params(W, H, 1.5, 1.5, N=32)
    prm.fsize = fsize
    eng, _ = make_engine(prm)
    rng = np.random.default_rng(fsize)
    U = (rng.normal(0, 4, size=(H, W)) + np.linspace(-8, 8, W)[None, :]).astype(np.float32)
    V = rng.normal(0, 4, size=(H, W)).astype(np.float32)
    I = random_image(rng, W, H)
    eng.write_buffer(bm.BM_BUF_FLOW_IN, np.concatenate([U.ravel(), V.ravel()]))
    d_I = _dev(I)
    eng.process(d_I.data_ptr())
    torch.cuda.synchronize()
    med = eng.read_buffer(bm.BM_BUF_FLOW_MED, np.float32).reshape(2, H, W)
    out = eng.read_buffer(bm.BM_BUF_FLOW_OUT, np.float32).reshape(2, H, W)
    Um, Vm, Uo, Vo = oracle.refine(U, V, I, fsize, prm.sEPE, prm.sI, prm.sS)
    assert np.array_equal(med[0], Um) and np.array_equal(med[1], Vm)
    err = max(np.abs(out[0] - Uo).max(), np.abs(out[1] - Vo).max())
    assert err <= FLOW_TOL, err


def _oracle_sequence(eng, prm, pattern, frames):
    """Run frames through the engine (bm_frame) and the oracle on the engine's
    up-sampled images and random stream; return both outputs per pair."""
    normals_cache = {}

    def normals_fn(call, n):
        if call not in normals_cache:
            normals_cache[call] = engine_normals(eng, call)
        return normals_cache[call]

    seq = oracle.Sequence(prm.as_dict(), pattern, normals_fn, nn=eng.nn_indices())
    results = []
    for k, f in enumerate(frames):
        d = _dev(f)
        u = torch.empty(prm.sy_in, prm.sx_in, device="cuda")
        v = torch.empty(prm.sy_in, prm.sx_in, device="cuda")
        eng.frame(d.data_ptr(), True, u.data_ptr(), v.data_ptr(), True)
        torch.cuda.synchronize()
        nx, ny, cost, _ = engine_field(eng)
        uv_in = eng.read_buffer(bm.BM_BUF_FLOW_IN, np.float32).reshape(2, prm.sy_in, prm.sx_in)
        d_up = torch.empty(prm.sy, prm.sx, device="cuda")
        eng.upsample_u8(d.data_ptr(), d_up.data_ptr())
        torch.cuda.synchronize()
        # without re-sampling the engine describes the frame itself, as the oracle does
        resampled = prm.sx != prm.sx_in or prm.sy != prm.sy_in
        o = seq.frame(f, up=d_up.cpu().numpy() if resampled else None)
        if k == 0:
            assert o is None
            assert float(u.abs().max()) == 0.0
            continue
        results.append(dict(u=u.cpu().numpy(), v=v.cpu().numpy(), nx=nx, ny=ny, cost=cost, uv_in=uv_in,
                            ou=o[0], ov=o[1], NX=seq.NX, NY=seq.NY, H=seq.H, U=seq.U, V=seq.V))
    return results


@pytest.mark.parametrize("W,H,u,N", [(96, 64, 1.5, 32), (80, 52, 2.9, 128), (70, 45, 4.9, 512), (64, 40, 1.0, 64)])
def test_pair_end_to_end(W, H, u, N):
    from briefmatch_gb300 import synth

    prm = small_params(W, H, u, u, N=N)
    eng, pattern = make_engine(prm, pattern_seed=W)
    f1, f2, _, _ = synth.make_pair(W, W, H, 6.0)
    (r,) = _oracle_sequence(eng, prm, pattern, [f1, f2])
    assert np.array_equal(r["nx"], r["NX"]) and np.array_equal(r["ny"], r["NY"])
    assert np.array_equal(r["cost"], r["H"])
    assert np.array_equal(r["uv_in"][0], r["U"]) and np.array_equal(r["uv_in"][1], r["V"])
    err = max(np.abs(r["u"] - r["ou"]).max(), np.abs(r["v"] - r["ov"]).max())
    assert err <= FLOW_TOL, err


def test_sequence_temporal_init():
    from briefmatch_gb300 import synth

    W, H = 88, 60
    prm = small_params(W, H, 2.0, 2.0, N=64)
    eng, pattern = make_engine(prm, pattern_seed=9)
    frames, _ = synth.make_sequence(5, W, H, 5, vmax=5.0)
    res = _oracle_sequence(eng, prm, pattern, frames)
    assert len(res) == 4
    for r in res:
        assert np.array_equal(r["nx"], r["NX"]) and np.array_equal(r["ny"], r["NY"])
        assert np.array_equal(r["cost"], r["H"])
        err = max(np.abs(r["u"] - r["ou"]).max(), np.abs(r["v"] - r["ov"]).max())
        assert err <= FLOW_TOL, err


def test_host_frames_and_determinism():
    from briefmatch_gb300 import synth

    W, H = 128, 96
    prm = small_params(W, H, 2.0, 2.0, N=128)
    outs = []
    for _ in range(2):
        eng = bm.FlowEngine(prm)
        f1, f2, ugt, vgt = synth.make_pair(11, W, H, 5.0)
        eng.process_frame(f1)
        outs.append(eng.process_frame(f2))
        eng.clean()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_errors_are_status_codes():
    prm = small_params(64, 48)
    eng, _ = make_engine(prm)
    with pytest.raises(bm.BriefMatchException):
        eng.set_pattern(np.zeros(3, np.float32))
    with pytest.raises(bm.BriefMatchException):
        eng.features(0, 1)
    with pytest.raises(bm.BriefMatchException):
        eng.features(1, 5)
