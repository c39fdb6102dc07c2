"""Build recipe of libawigner.so (sm_103a), in-tree.

The translation units are compiled in parallel with nvcc for sm_103a and
linked into ``accuratewigner_gb300/libawigner.so``; NVRTC (dynamic) compiles
the user-expression modules at run time.  Objects go to ``_build/`` at the
repository root.  Rebuilds only what is out of date.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libawigner.so")

# the double-float pass kernels are the slowest to compile: one unit per line length, started first
DF_SIZES = [32, 64, 128, 256, 512, 1024, 2048, 4096, 8192]
SOURCES = (["aw_pass_df_%d.cu" % n for n in DF_SIZES] +
           ["aw_api.cu", "aw_util.cu", "aw_pass_f64.cu", "aw_pass_f32.cu", "aw_pass_df.cu", "aw_noalloc.cu"])
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc():
    cand = os.path.join(CUDA_HOME, "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _stale(target, inputs):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(i) > t for i in inputs)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + deps):
            jobs.append([_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                            "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    sys.stderr.write(out)
    if force or jobs or _stale(LIB, objs):
        libdir = os.path.join(CUDA_HOME, "lib64")
        _run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-L" + libdir, "-lnvrtc", "-Xlinker", "-rpath=" + libdir])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
