"""CPU checks of the C ABI: the library loads, exports every entry point the header
declares, and its host-only parameter logic follows the reference."""
from __future__ import annotations

import ctypes
import math
import os
import re

import numpy as np
import pytest

import briefmatch_gb300 as bm
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names.update(re.findall(r"^\s*(?:[\w\s\*]+?)\b(bm_\w+)\s*\(", txt, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(bm.LIB_PATH)
    names = _declared_symbols()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version():
    assert "sm_103a" in bm.version()


def test_params_default_match_reference():
    # briefmatch.h:67-84
    p = bm.BMParams()
    assert (p.sx, p.sy, p.sx_in, p.sy_in) == (64, 64, 64, 64)
    assert (p.iterations, p.jfMax, p.P, p.fsize, p.N) == (2, 256, 11, 13, 128)
    assert (p.doubleProp, p.filter, p.tInit) == (1, 1, 1)
    assert p.sigma == np.float32(0.5) and p.patchArea == 75 and p.sS == 6
    assert p.sEPE == np.float32(0.4) and p.sI == np.float32(0.1) and p.maxmot == 5


@pytest.mark.parametrize("W,H,u,grid,patch,fsize,sS", [
    (584, 388, 1.5, (876, 582), 31.55, 9, 5.96),
    (1024, 436, 2.9, (2969, 1264), 96.8, 13, 9.46),
    (1920, 1080, 4.9, (9408, 5292), 323.8, 23, 18.7),
    (512, 384, 2.9, (1484, 1113), 55.7, 7, 5.44),
])
def test_derivation_matches_workload_table(W, H, u, grid, patch, fsize, sS):
    # of_pipeline.cpp:178-190
    p = bm.BMParams.derive(W, H, u, u)
    assert (p.sx, p.sy) == grid
    assert abs(p.patchArea - patch) < 0.06
    assert p.fsize == fsize
    assert abs(p.sS - sS) < 0.03  # the table rounds to 3 significant figures
    diag_up = math.sqrt(p.sx ** 2 + p.sy ** 2)
    assert abs(p.sigma - 0.00025 * diag_up) < 1e-3


def test_derivation_defaults_for_unset_factors():
    p = bm.BMParams.derive(100, 50)
    assert (p.sx, p.sy) == (int(np.float32(2.740) * 100), int(np.float32(3.052) * 50))


def test_pattern_properties():
    p = bm.BMParams.derive(1024, 436, 2.9, 2.9, N=128)
    a = p.make_pattern(1)
    b = p.make_pattern(1)
    c = p.make_pattern(2)
    assert a.shape == (512,) and np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.abs(a).max() <= p.patchArea
    # sign(g) g^2 with g ~ N(0, 0.2): E|.| = 0.04 * patchArea
    assert 0.025 * p.patchArea < np.abs(a).mean() < 0.055 * p.patchArea


def test_gauss_taps_match_oracle():
    for sigma in (0.263, 0.807, 2.70, 5.0, 16.0):
        p = bm.BMParams(sigma=sigma)
        t = p.gauss_taps()
        assert t.size == int(math.ceil(np.float32(sigma) * 3)) * 2 + 1
        assert np.array_equal(t, oracle.gauss_taps(np.float32(sigma)))
        assert abs(float(t.sum()) - 1.0) < 1e-5


def _create(**kw):
    p = bm.BMParams(**kw)
    ctx = ctypes.c_void_p()
    return bm.lib().bm_create(ctypes.byref(p.struct()), ctypes.byref(ctx)), ctx


@pytest.mark.parametrize("kw,msg", [
    (dict(N=513), "Feature length exceeds"),
    (dict(fsize=49), "Median filter size exceeds"),
    (dict(sigma=17.0), "Gaussian down-sampling filter"),
    (dict(sx=40000, sy=10), "int16"),
])
def test_limits_rejected_before_any_allocation(kw, msg):
    # briefmatch.cpp:78-96: the limits are checked before touching the device
    st, ctx = _create(**kw)
    assert st == bm.BM_ERR_LIMIT
    assert msg in bm.lib().bm_last_error().decode()
    assert not ctx.value


def test_null_arguments():
    L = bm.lib()
    assert L.bm_create(None, None) == bm.BM_ERR_INVALID
    assert L.bm_params_default(None) == bm.BM_ERR_INVALID
    assert L.bm_frame(None, None, 0, None, None, 0) == bm.BM_ERR_INVALID
    assert L.bm_destroy(None) == bm.BM_OK
    assert L.bm_launch_count(None) == 0


@pytest.mark.parametrize("w,h,u,N", [(584, 388, 1.5, 32), (1024, 436, 2.9, 128), (1920, 1080, 4.9, 512),
                                     (512, 384, 2.9, 128), (77, 53, 2.0, 64), (640, 480, 0.0, 128)])
def test_oracle_parameters_and_pattern_equal_the_engine(w, h, u, N):
    """The oracle derives parameters (of_pipeline.cpp:178-190) and draws the pattern
    (briefmatch.cpp:124-148) on its own, so that the bench's reference arm needs no
    engine library; both restatements give the same values."""
    e = bm.BMParams.derive(w, h, u, u, N=N)
    o = oracle.derive_params(w, h, u, u, N=N)
    ed = e.as_dict()
    assert set(ed) == set(o)
    for k in ed:
        assert np.float32(ed[k]) == np.float32(o[k]), (k, ed[k], o[k])
    assert np.array_equal(e.make_pattern(99), oracle.make_pattern(o, 99))
    assert np.array_equal(e.gauss_taps(), oracle.gauss_taps(o["sigma"]))
