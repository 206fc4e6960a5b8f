"""Builds libdgcu.so in-tree (hopefoam_gb300/lib/) with nvcc for sm_103a.

Translation units compile in parallel; the result is a plain C-ABI shared
library (include/dgcu.h) loaded by ctypes."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libdgcu.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "-I" + CSRC,
          "-I" + os.path.join(HERE, "..", "include")]

SOURCES = ["dg_api.cu", "euler_fp64.cu", "euler_split.cu", "euler_split_pipe.cu", "euler_noalloc.cu", "ipdg.cu", "ipdg_api.cu", "lpc.cu", "schwarz_tc.cu", "schwarz_mlp.cu", "batch_api.cu", "ins.cu", "mg.cu", "limiter.cu",
           "dg_basis.cpp"]


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src.replace(".", "_") + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "dgcu.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + COMMON + ["-c", path, "-o", obj]
    else:
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", path, "-o", obj]
    extra = os.environ.get("DGCU_NVCC_FLAGS")
    if extra:
        cmd += extra.split()
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
