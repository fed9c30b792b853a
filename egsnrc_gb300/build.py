"""Build step: compiles the CUDA engine (libegsgpu.so, sm_103a) in-tree and,
optionally, the FP64 CPU oracle used by the tests.

    python -m egsnrc_gb300.build            # engine + oracle
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libegsgpu.so")
APP = os.path.join(HERE, "egs_gpu_app")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--use_fast_math"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_engine(force=False):
    srcs = [os.path.join(CSRC, f) for f in ("egs_transport.cu", "egs_hatch.cpp", "egs_transport_f64.cu", "egs_phsp.cpp")]
    deps = srcs + [os.path.join(CSRC, f) for f in ("egs_device.cuh", "egs_physics.cuh", "egs_hatch.h")] + [
        os.path.join(ROOT, "include", "egsgpu.h")]
    if not force and _newer(LIB, deps):
        return LIB
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    objs = [os.path.join(bdir, "egs_transport.o"), os.path.join(bdir, "egs_hatch.o"),
            os.path.join(bdir, "egs_transport_f64.o"), os.path.join(bdir, "egs_phsp.o")]
    cmds = [
        [NVCC] + ARCH + NVFLAGS + ["-c", srcs[0], "-o", objs[0]],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-c", srcs[1], "-o", objs[1]],
        # the FP64 engine rounds like the CPU oracle: no fused multiply-adds
        [NVCC] + ARCH + NVFLAGS + ["--fmad=false", "-c", srcs[2], "-o", objs[2]],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-c", srcs[3], "-o", objs[3]],
    ]
    with ThreadPoolExecutor(4) as ex:
        list(ex.map(_run, cmds))
    _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_app(force=False):
    src = os.path.join(CSRC, "egs_gpu_app.cpp")
    if not os.path.exists(src):
        return None
    deps = [src, os.path.join(CSRC, "egs_input.h"), LIB]
    if not force and _newer(APP, deps):
        return APP
    _run(["g++", "-O2", "-std=c++17", "-o", APP, src, "-I" + os.path.join(ROOT, "include"),
          "-L" + HERE, "-legsgpu", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + HERE])
    return APP


def reference_dir():
    """The reference checkout used to build oracle/_ref, or None."""
    for d in (os.environ.get("EGSNRC_REFERENCE"), "/root/reference"):
        if d and os.path.isdir(os.path.join(d, "HEN_HOUSE")):
            return d
    return None


def build_oracle(force=False):
    if force:
        for f in (ORACLE_LIB, os.path.join(ORACLE_DIR, "liboracle_fast.so")):
            if os.path.exists(f):
                os.remove(f)
    _run(["make", "-s", "-j2", "all"], cwd=ORACLE_DIR)
    # the reference's own code that compiles standalone (oracle/_ref), where
    # its sources are present: EGSNRC_REFERENCE names the checkout (the
    # directory holding HEN_HOUSE)
    ref = reference_dir()
    if ref:
        _run(["make", "-s", "ref", "REF=" + ref], cwd=ORACLE_DIR)
    return ORACLE_LIB


def build_all(force=False):
    build_engine(force)
    build_oracle(force)
    build_app(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
