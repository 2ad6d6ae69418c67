"""The briefmatch command line: option handling and frame reading (no GPU needed;
these paths end before the engine is set up)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from briefmatch_gb300 import build as b
from pngio import write_pgm, write_png

CLI = b.CLI


@pytest.fixture(scope="module", autouse=True)
def _cli():
    b.build_cli()
    assert os.path.exists(CLI)


def run(*args):
    p = subprocess.run([CLI, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=60)
    return p.returncode, p.stdout, p.stderr


def test_help_lists_every_reference_option():
    rc, out, _ = run("-h")
    assert rc == 1  # main.cpp:52-53: setParams returns false after the help text
    for opt in ("--input", "--output", "--frames", "--vis-max-motion", "--verbose", "--feature-length",
                "--patch-radius", "--up-sampling-x", "--up-sampling-y", "--sigma-downsampling", "--iterations",
                "--jf-max", "--median-size", "--range-epe", "--range-i", "--range-spatial", "--flow-gt"):
        assert opt in out


def test_help_lists_the_engine_options():
    """Options the engine adds to the reference's: random stream, pattern seed, and the
    learned proposal with its schedule and input reduction."""
    rc, out, _ = run("-h")
    assert rc == 1
    for opt in ("--random-stream", "--pattern-seed", "--proposal", "--proposal-iterations", "--proposal-jf-max",
                "--proposal-local-steps", "--proposal-reduce"):
        assert opt in out


@pytest.mark.parametrize("args,msg", [
    ((), "Missing required option '--input'"),
    (("-i", "x.pgm", "-fl", "600"), "Valid range is [2, 512]"),
    (("-i", "x.pgm", "-ux", "0.5"), "out of range"),
    (("-i", "x.pgm", "--bogus"), "'--bogus' is not a valid input option"),
    (("-i",), "No value provided for input option '-i'"),
    (("-i", "x.pgm", "-o", "out.jpg"), "Unsupported output format"),
    (("-i", "x.pgm", "-f", "3"), "Unable to parse frame range"),
    (("-i", "x.pgm", "-f", "5:2"), "End frame should be >= start frame"),
    (("-i", "x.pgm", "-rng", "mt"), "not valid"),
    (("-i", "x.pgm", "--proposal-reduce", "8"), "out of range"),
])
def test_parser_errors(args, msg):
    rc, _, err = run(*args)
    assert rc == 1
    assert "briefmatch input error" in err and msg in err


def test_missing_frame_is_a_briefmatch_error(tmp_path):
    rc, _, err = run("-i", str(tmp_path / "frame%02d.pgm"), "-f", "1:3")
    assert rc == 1 and "briefmatch error: Cannot read image file" in err


@pytest.mark.parametrize("fmt", ["pgm", "png"])
def test_reads_first_frame_size(tmp_path, fmt):
    img = (np.arange(37 * 23) % 256).astype(np.uint8).reshape(23, 37)
    path = tmp_path / ("frame%02d." + fmt)
    (write_pgm if fmt == "pgm" else write_png)(str(path).replace("%02d", "01"), img)
    rc, out, err = run("-i", str(path), "-f", "1:1", "-v")
    # without a GPU the run stops at engine set-up; the frame was read and sized
    assert "Image resolution:        37x23" in err
