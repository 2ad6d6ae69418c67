"""Build recipe for the engine library (sm_103a) and, for the tests, the CPU oracle.

Everything is compiled in-tree with nvcc/gcc directly (no cmake), translation
units in parallel:

  briefmatch_gb300/_lib/libbriefmatch_gb300.so   engine (CUDA kernels + C ABI)
  briefmatch_gb300/_lib/briefmatch                command line (C++ BriefMatch/OFPipeline)
  oracle/_build/libbmoracle.so                    CPU restatement (test infrastructure)
  oracle/_build/librefshim.so                     loader for the reference kernel build
  oracle/_ref/*.cubin                             reference kernels compiled from their
                                                  own sources (only where those exist)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "briefmatch_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libbriefmatch_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libbmoracle.so")
REFSHIM_LIB = os.path.join(ORACLE_BUILD, "librefshim.so")
REF_OUT = os.path.join(ORACLE_DIR, "_ref")
# Where the reference's sources are read from (build_reference), if present there:
# the environment variable BM_REFERENCE_ROOT, else the read-only checkout this recipe
# was written against.
REFERENCE_ROOT = os.environ.get("BM_REFERENCE_ROOT", "/root/reference")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# (source, extra flags).  The kernel unit uses the reference's -use_fast_math so the
# expressions whose rounding the reference fixes compile to the same instructions.
ENGINE_UNITS = [
    ("bm_kernels.cu", ["-use_fast_math", "-Xptxas", "-v"]),
    ("bm_batch.cu", ["-use_fast_math"]),
    ("bm_api.cu", []),
    ("bm_noalloc.cu", []),
    ("bm_color.cu", []),
    ("bm_net.cu", []),
    ("bm_params.cpp", []),
    ("bm_alloc.cpp", []),
]


def _run(cmd, cwd=ROOT):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _newer(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    return hs


def build_engine(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src, extra in ENGINE_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            if src.endswith(".cpp"):
                cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                       "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o]
            else:
                cmd = [NVCC] + NVCC_COMMON + extra + ["-c", s, "-o", o]
            jobs.append(cmd)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


CXX_DIR = os.path.join(CSRC, "cxx")
CXX_UNITS = ["briefmatch.cpp", "of_pipeline.cpp", "flow_io.cpp", "main.cpp"]
CLI = os.path.join(LIBDIR, "briefmatch")


def _have_zlib():
    probe = os.path.join(BUILD, "zprobe.c")
    with open(probe, "w") as f:
        f.write("#include <zlib.h>\nint main(void){return (int)zlibVersion()[0] == 0;}\n")
    p = subprocess.run(["gcc", probe, "-lz", "-o", os.path.join(BUILD, "zprobe")], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT)
    return p.returncode == 0


def build_cli(force=False):
    """The briefmatch command line: the reference's BriefMatch/OFPipeline API (C++)
    over the engine library, linked with rpath $ORIGIN.  PNG I/O needs zlib; without
    it the CLI reads PGM/PPM and writes .flo/.bin only."""
    os.makedirs(BUILD, exist_ok=True)
    zlib = _have_zlib()
    srcs = [os.path.join(CXX_DIR, u) for u in CXX_UNITS]
    hdrs = [os.path.join(CXX_DIR, f) for f in os.listdir(CXX_DIR) if f.endswith(".h")] + _headers()
    if not (force or _newer(CLI, srcs + hdrs + [LIB])):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CXX_DIR]
    if zlib:
        cmd.append("-DBM_HAVE_ZLIB")
    cmd += srcs + ["-o", CLI, "-L" + LIBDIR, "-lbriefmatch_gb300", "-Wl,-rpath,$ORIGIN"]
    if zlib:
        cmd.append("-lz")
    _run(cmd)
    return CLI


def build_oracle(force=False):
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE_DIR, "bm_oracle.c")
    src_pat = os.path.join(ORACLE_DIR, "bm_oracle_params.cpp")
    if force or _newer(ORACLE_LIB, [src, src_pat, os.path.join(ORACLE_DIR, "bm_oracle.h")]):
        obj_c = os.path.join(ORACLE_BUILD, "bm_oracle.o")
        obj_p = os.path.join(ORACLE_BUILD, "bm_oracle_params.o")
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-c", src, "-o", obj_c])
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src_pat, "-o", obj_p])
        _run(["g++", "-shared", "-fopenmp", "-o", ORACLE_LIB, obj_c, obj_p, "-lm"])
    shim = os.path.join(ORACLE_DIR, "refshim.c")
    if os.path.exists(shim) and (force or _newer(REFSHIM_LIB, [shim])):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-I" + os.path.join(CUDA_HOME, "include"), "-o",
              REFSHIM_LIB, shim, "-ldl"])
    return ORACLE_LIB


def build_reference(ref_root=None, force=False):
    """Compile the reference's own kernel sources, unmodified, to sm_103a cubins.

    The reference's host code needs OpenCV, Boost and libpng (absent), so only its
    two kernel units are built, with its own nvcc flags (-O3 -use_fast_math).  The
    cubins land in oracle/_ref and are loaded by oracle/refshim.c on the GPU.
    Returns the list of cubins, or [] when the reference sources are not present.
    """
    kdir = os.path.join(ref_root or REFERENCE_ROOT, "kernels")
    if not os.path.isdir(kdir):
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    outs = []
    jobs = []
    for unit in ("briefmatch_cuda", "util_cuda"):
        src = os.path.join(kdir, unit + ".cu")
        out = os.path.join(REF_OUT, unit + ".cubin")
        outs.append(out)
        if force or _newer(out, [src]):
            jobs.append([NVCC, "-cubin"] + ARCH + ["-O3", "-use_fast_math", "-Wno-deprecated-gpu-targets", "-I" + kdir,
                                                   src, "-o", out])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    return outs


def build_all(force=False, verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_engine, force, verbose)
        f2 = ex.submit(build_oracle, force)
        f3 = ex.submit(build_reference, None, force)
        lib = f1.result()
        cli = build_cli(force)
        return lib, cli, f2.result(), f3.result()


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
