"""The briefmatch command line end to end on the GPU: frames from PNG/PGM files,
flow written as .flo/.bin/.png, identical to the library path."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import briefmatch_gb300 as bm
from briefmatch_gb300 import build as b
from briefmatch_gb300 import synth
from pngio import read_flo, read_png_rgb, write_flo, write_pgm, write_png

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)


def run(*args):
    b.build_cli()
    p = subprocess.run([b.CLI, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    return p.stdout


@pytest.mark.parametrize("fmt", ["png", "pgm"])
def test_cli_flo_matches_library(tmp_path, fmt):
    W, H = 120, 80
    frames, flows = synth.make_sequence(3, W, H, 4, vmax=5.0)
    for k, f in enumerate(frames):
        (write_png if fmt == "png" else write_pgm)(str(tmp_path / ("f%02d." % k + fmt)), f)
    run("-i", str(tmp_path / ("f%02d." + fmt)), "-f", "0:3", "-o", str(tmp_path / "o%02d.flo"), "-ux", "2", "-uy",
        "2", "-fl", "64")
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    eng = bm.FlowEngine(prm)
    for k, f in enumerate(frames):
        u, v = eng.process_frame(f)
        fu, fv = read_flo(str(tmp_path / ("o%02d.flo" % k)))
        assert np.array_equal(fu, u) and np.array_equal(fv, v), k
    eng.clean()


def test_cli_bin_png_and_epe(tmp_path):
    W, H = 96, 64
    frames, flows = synth.make_sequence(4, W, H, 2, vmax=4.0)
    for k, f in enumerate(frames):
        write_png(str(tmp_path / ("f%02d.png" % k)), f)
    write_flo(str(tmp_path / "gt.flo"), *flows[0])
    out = run("-i", str(tmp_path / "f%02d.png"), "-f", "0:1", "-o", str(tmp_path / "o%02d.bin"), "-gt",
              str(tmp_path / "gt.flo"))
    epe_lines = [l for l in out.splitlines() if l.startswith("Error (EPE)")]
    assert len(epe_lines) == 1 and 0 <= float(epe_lines[0].split("=")[1]) < 10
    raw = np.fromfile(str(tmp_path / "o01.bin"), np.float32)
    assert raw.size == 2 * W * H and np.isfinite(raw).all()
    # the colour PNG (briefmatch.cpp:373-421, colorcode.cpp:52-74; coloured on the GPU)
    # equals the oracle's colour coding of the same flow, byte for byte, with a fixed
    # and with the measured motion range
    import oracle

    run("-i", str(tmp_path / "f%02d.png"), "-f", "0:1", "-o", str(tmp_path / "o%02d.flo"))
    fu, fv = read_flo(str(tmp_path / "o01.flo"))
    # no -mm: BMParams' default maxmot (5, briefmatch.h:83); -mm 0: the measured range
    for mm, extra in ((5.0, []), (2.5, ["-mm", "2.5"]), (0.0, ["-mm", "0"])):
        run("-i", str(tmp_path / "f%02d.png"), "-f", "0:1", "-o", str(tmp_path / "c%02d.png"), *extra)
        rgb = read_png_rgb(str(tmp_path / "c01.png"))
        assert rgb.shape == (H, W, 3) and rgb.std() > 0
        assert np.array_equal(rgb, oracle.flow_colors(fu, fv, mm)), mm


@pytest.mark.parametrize("reduce", [1, 2])
def test_cli_proposal_matches_library(tmp_path, reduce):
    """--proposal seeds every pair with the learned proposal, as bm_set_proposal does
    (--proposal-reduce as bm_set_proposal_reduce)."""
    from briefmatch_gb300 import learn

    W, H = 120, 80
    frames, _ = synth.make_sequence(5, W, H, 3, vmax=6.0)
    for k, f in enumerate(frames):
        write_pgm(str(tmp_path / ("f%02d.pgm" % k)), f)
    run("-i", str(tmp_path / "f%02d.pgm"), "-f", "0:2", "-o", str(tmp_path / "o%02d.flo"), "-ux", "2", "-uy", "2",
        "-fl", "64", "--proposal", learn.DEFAULT_WEIGHTS, "-pit", "1", "-pjm", "8", "-pls", "2",
        "--proposal-reduce", str(reduce))
    prm = bm.BMParams.derive(W, H, 2.0, 2.0, N=64)
    eng = bm.FlowEngine(prm)
    net = learn.load_net(learn.DEFAULT_WEIGHTS, 1, H // 4, W // 4)
    bm.set_proposal(eng, net, 0.5, 1, 8)
    bm.set_local_steps(eng, 2, 2)
    bm.set_proposal_reduce(eng, reduce)
    for k, f in enumerate(frames):
        u, v = eng.process_frame(f)
        fu, fv = read_flo(str(tmp_path / ("o%02d.flo" % k)))
        assert np.array_equal(fu, u) and np.array_equal(fv, v), k
    eng.clean()
    with pytest.raises(AssertionError):
        run("-i", str(tmp_path / "f%02d.pgm"), "-f", "0:1", "--proposal", str(tmp_path / "f00.pgm"))
