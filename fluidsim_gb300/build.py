"""Build libfluidsim_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel into _build/, then linked.
No CMake, no torch extension machinery: the library is a plain C-ABI shared
object that depends only on the CUDA runtime.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "libfluidsim_gb300.so")
SOURCES = ["fs_api.cu", "fs_ptcl.cu", "fs_lapl.cu", "fs_mixed.cu", "fs_lapl_mixed.cu", "fs_lpc.cu", "fs_conv_tc.cu", "fs_probe.cu", "fs_host.cpp", "fs_batch.cpp", "fs_output.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _flags(src):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "-Xptxas", "-warn-spills"]
    return common


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    s = os.path.join(CSRC, src)
    deps = [s] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "fluidsim_gpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc(), "-c", s, "-o", obj] + _flags(src)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr if verbose else ""


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in res]
    for _, log in res:
        if log:
            sys.stderr.write(log)
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(o) for o in objs):
        return OUT
    cmd = [nvcc(), "-shared", "-o", OUT] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
