"""Build icep_kapsel_gb300/libicep_gb300.so (in-tree) for sm_103a.

Each CUDA translation unit under csrc/ is compiled by its own nvcc process
(in parallel), then linked into one shared library with the CUDA runtime
linked statically; the command-line driver icep_kapsel_gb300/icep_kapsel
(csrc/kapsel_main.cpp) links against it. Objects go to
icep_kapsel_gb300/_build/.

    python -m icep_kapsel_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libicep_gb300.so")
BIN = os.path.join(HERE, "icep_kapsel")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["fft_df.cu", "fft.cu", "fields.cu", "particles.cu", "krylov.cu", "kspace.cu", "kop.cu", "unet.cu", "engine.cu", "icep_abi.cu", "lj_noalloc.cu", "probe.cu", "refine.cu", "solve_graph.cu", "udf.cu", "avs.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_dep():
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def build(force=False, verbose=False):
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_dep() and os.path.exists(BIN)
            and os.path.getmtime(BIN) >= _newest_dep()):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nv] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    # the command-line driver (kapsel -I input.udf), linked against the library
    main = os.path.join(CSRC, "kapsel_main.cpp")
    tmpb = BIN + ".tmp"
    cmd = [nv, "-O2", "-std=c++17", main, "-o", tmpb, "-L" + HERE, "-licep_gb300", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmpb, BIN)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
