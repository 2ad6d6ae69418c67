"""Golden vectors from the reference's own kernels.

Runs the reference kernel layer (kernels/briefmatch_cuda.cu and util_cuda.cu
compiled unmodified to oracle/_ref/*.cubin, launched through oracle/refshim) on
small seeded inputs and stores inputs and outputs in tests/golden/*.npz, so that
the CPU tests can pin the oracle without a GPU.  Needs a GPU and the prebuilt
oracle/_ref cubins; the engine library supplies the two device-side tables the
oracle takes as inputs (the random-search normals of the reference's curand
stream and the resizeNN index tables, see oracle/__init__.py).

  python tests/golden/make_golden.py [output_dir]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def main(out_dir):
    import torch

    import briefmatch_gb300 as bm
    from bmtest import random_field, random_image
    from briefmatch_gb300 import synth
    from oracle import refshim

    if not refshim.available():
        raise SystemExit("reference kernel build (oracle/_ref) not present")
    ref = refshim.RefKernels()
    os.makedirs(out_dir, exist_ok=True)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    # 1. Lanczos up-sampling (util_cuda.cu:126-158)
    out = {}
    for k, (W, H, u) in enumerate([(37, 23, 2.9), (40, 30, 1.5), (21, 17, 4.9)]):
        img = random_image(np.random.default_rng(100 + k), W, H)
        prm = bm.BMParams.derive(W, H, u, u)
        d = dev(img)
        o = torch.empty(prm.sy, prm.sx, device="cuda")
        ref.resize_lanczos(d.data_ptr(), o.data_ptr(), W, H, prm.sx, prm.sy)
        torch.cuda.synchronize()
        out["in%d" % k] = img
        out["out%d" % k] = o.cpu().numpy()
    np.savez_compressed(os.path.join(out_dir, "upsample.npz"), **out)

    # 2. BRIEF descriptors (briefmatch_cuda.cu:82-124), N = 32, 100, 512
    out = {}
    for N, (W, H) in ((32, (64, 48)), (100, (48, 40)), (512, (40, 32))):
        prm = bm.BMParams.derive(W, H, 1.0, 1.0, N=N)
        pattern = prm.make_pattern(N)
        img = random_image(np.random.default_rng(N), W, H)
        ref.set_pattern(pattern)
        ns = (N + 31) // 32
        F = torch.zeros(W * H * ns, dtype=torch.int32, device="cuda")
        d = dev(img)
        ref.binary_features(d.data_ptr(), F.data_ptr(), W, H, N, ns)
        torch.cuda.synchronize()
        out["img_N%d" % N] = img
        out["pattern_N%d" % N] = pattern
        out["F_N%d" % N] = F.cpu().numpy().view(np.uint32).reshape(W * H, ns)
    np.savez_compressed(os.path.join(out_dir, "features.npz"), **out)

    # 3. zero initialisation + three random searches (briefmatch_cuda.cu:149-246)
    W, H, N = 72, 52, 128
    prm = bm.BMParams.derive(W, H, 1.0, 1.0, N=N)
    pattern = prm.make_pattern(5)
    ref.set_pattern(pattern)
    f1, f2, _, _ = synth.make_pair(5, W, H, 6.0)
    ns = N // 32
    n = W * H
    Fs = []
    for img in (f1.astype(np.float32), f2.astype(np.float32)):
        F = torch.zeros(n * ns, dtype=torch.int32, device="cuda")
        d = dev(img)
        ref.binary_features(d.data_ptr(), F.data_ptr(), W, H, N, ns)
        Fs.append(F)
    guard = (prm.jfMax + 1) * W + prm.jfMax
    _, NX = refshim.guarded(torch, n, guard, torch.int16)
    _, NY = refshim.guarded(torch, n, guard, torch.int16)
    D = torch.zeros(n, device="cuda")
    state = torch.zeros(n * refshim.CURAND_STATE_BYTES, dtype=torch.uint8, device="cuda")
    ref.init_random(state.data_ptr(), W, H)
    ref.initialize(Fs[0].data_ptr(), Fs[1].data_ptr(), D.data_ptr(), NX.data_ptr(), NY.data_ptr(), W, H, True, N, ns)
    torch.cuda.synchronize()
    out = {"F1": Fs[0].cpu().numpy().view(np.uint32).reshape(n, ns), "F2": Fs[1].cpu().numpy().view(np.uint32).reshape(n, ns),
           "NX_init": NX.cpu().numpy(), "NY_init": NY.cpu().numpy(), "D_init": D.cpu().numpy(),
           "dist": np.float32(prm.search_dist())}
    eng = bm.BriefMatch(prm)
    eng.setup()
    for call in range(3):
        nrm = torch.empty(2 * n, device="cuda")
        eng.normals(call, nrm.data_ptr())
        ref.random_search(Fs[0].data_ptr(), Fs[1].data_ptr(), D.data_ptr(), NX.data_ptr(), NY.data_ptr(),
                          state.data_ptr(), W, H, prm.search_dist(), N, ns)
        torch.cuda.synchronize()
        out["normals%d" % call] = nrm.cpu().numpy()
        out["NX_rs%d" % call] = NX.cpu().numpy()
        out["NY_rs%d" % call] = NY.cpu().numpy()
        out["D_rs%d" % call] = D.cpu().numpy()
    eng.clean()
    np.savez_compressed(os.path.join(out_dir, "match.npz"), **out)

    # 4. down-sampling chain (briefmatch.cpp:296-324 + util_cuda.cu)
    W, H = 60, 40
    prm = bm.BMParams.derive(W, H, 2.9, 2.9, N=32)
    eng = bm.BriefMatch(prm)
    eng.setup()
    xs, ys = eng.nn_indices()
    eng.clean()
    NXf, NYf = random_field(np.random.default_rng(8), prm.sx, prm.sy, 20)
    taps = prm.gauss_taps()
    ref.set_kernel(taps)
    n = prm.sx * prm.sy
    out = {"NX": NXf, "NY": NYf, "taps": taps, "nnx": xs, "nny": ys,
           "dims": np.array([prm.sx, prm.sy, W, H], np.int32)}
    for comp, field, m in ((0, NXf, np.float32(W) / np.float32(prm.sx)), (1, NYf, np.float32(H) / np.float32(prm.sy))):
        src = dev(field)
        XF = torch.zeros(n, device="cuda")
        tmp = torch.zeros(n, device="cuda")
        XI = torch.zeros(W * H, device="cuda")
        ref.convert(src.data_ptr(), XF.data_ptr(), prm.sx, prm.sy)
        ref.filter_const(XF.data_ptr(), tmp.data_ptr(), taps.size, 1, prm.sx, prm.sy)
        ref.filter_const(tmp.data_ptr(), XF.data_ptr(), taps.size, 0, prm.sx, prm.sy)
        ref.resize_nn(XF.data_ptr(), XI.data_ptr(), prm.sx, prm.sy, W, H)
        ref.mult(XI.data_ptr(), float(m), W, H)
        torch.cuda.synchronize()
        out["UV"[comp]] = XI.cpu().numpy().reshape(H, W)
    np.savez_compressed(os.path.join(out_dir, "downsample.npz"), **out)

    # 5. median (util_cuda.cu:75-111) and cross-trilateral filter (briefmatch_cuda.cu:248-297)
    out = {}
    W, H = 61, 43
    prm = bm.BMParams.derive(W, H, 1.5, 1.5, N=32)
    sS = 6.0   # a 30x30 window (s = 15), wider than this frame size derives
    for fsize in (9, 13):
        rng = np.random.default_rng(fsize + 100)
        U = (rng.normal(0, 4, size=(H, W)) + np.linspace(-8, 8, W)[None, :]).astype(np.float32)
        V = rng.normal(0, 4, size=(H, W)).astype(np.float32)
        I = random_image(rng, W, H)
        n = W * H
        guard = (fsize // 2 + 1) * W + fsize
        meds = []
        for A in (U, V):
            _, src = refshim.guarded(torch, n, guard, torch.float32)
            _, tmp = refshim.guarded(torch, n, guard, torch.float32)
            dst = torch.zeros(n, device="cuda")
            src.copy_(torch.from_numpy(A.ravel()))
            ref.median(src.data_ptr(), tmp.data_ptr(), 1, fsize, W, H)
            ref.median(tmp.data_ptr(), dst.data_ptr(), 0, fsize, W, H)
            meds.append(dst)
        dU, dV, dI = dev(U), dev(V), dev(I)
        Uo = torch.zeros(n, device="cuda")
        Vo = torch.zeros(n, device="cuda")
        ref.cb_filter(dU.data_ptr(), dV.data_ptr(), Uo.data_ptr(), Vo.data_ptr(), meds[0].data_ptr(),
                      meds[1].data_ptr(), dI.data_ptr(), prm.sEPE * prm.sEPE, prm.sI * prm.sI, sS * sS, W, H)
        torch.cuda.synchronize()
        k = "_f%d" % fsize
        out.update({"U" + k: U, "V" + k: V, "I" + k: I, "Um" + k: meds[0].cpu().numpy().reshape(H, W),
                    "Vm" + k: meds[1].cpu().numpy().reshape(H, W), "Uo" + k: Uo.cpu().numpy().reshape(H, W),
                    "Vo" + k: Vo.cpu().numpy().reshape(H, W),
                    "sigmas" + k: np.array([prm.sEPE, prm.sI, sS], np.float32)})
    np.savez_compressed(os.path.join(out_dir, "refine.npz"), **out)
    print("golden vectors written to", out_dir)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
