"""bench.py's roofline bookkeeping on the CPU: the committed DRAM traffic figures
apply only to the workload they were captured on, and the algorithmic bytes per
launch follow the per-pixel figures of the kernels."""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import briefmatch_gb300 as bm  # noqa: E402


def test_traffic_only_on_its_workload():
    try:
        bench.set_config("2")
        t = bench.ncu_traffic("jump_level")
        assert t is not None and t > 0
        assert bench.ncu_traffic("no_such_kernel") is None
        for other in ("1", "3"):
            bench.set_config(other)
            assert bench.ncu_traffic("jump_level") is None
    finally:
        bench.set_config("2")


def test_algorithmic_bytes_per_pixel():
    prm = bm.BMParams.derive(1024, 436, 2.9, 2.9, N=128)
    n = prm.sx * prm.sy
    # own descriptor + gathered descriptor footprint (16 B each), field and cost read
    # and written: 44 B per up-sampled pixel and level at N128
    assert bench.algorithmic_bytes("jump_level", prm) == 44 * n
    assert bench.algorithmic_bytes("features", prm) == 20 * n
    assert bench.algorithmic_bytes("trilateral", prm) == 28 * prm.sx_in * prm.sy_in
