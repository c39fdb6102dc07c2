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

# The pass kernels of each arithmetic form and line length compile in a unit of their own, generated
# into _build/gen/ (an include of aw_pass.cuh and one AW_SIZE_LAUNCHERS line), largest first.
SIZES = [8192, 4096, 2048, 1024, 512, 256, 128, 64, 32]
FORMS = [("df", "dfc"), ("f64", "double2"), ("f32", "float2")]
SOURCES = ["aw_api.cu", "aw_util.cu", "aw_pass_dispatch.cu", "aw_noalloc.cu"]
GEN = os.path.join(BUILD, "gen")


def _generated():
    """(path, text) of every generated pass unit."""
    out = []
    for n in SIZES:
        for tag, vt in FORMS:
            text = "// generated by _build.py: %s pass kernels of line length %d\n" % (tag, n)
            text += '#include "aw_pass.cuh"\n\nAW_SIZE_LAUNCHERS(%s, %s, %d)\n' % (vt, tag, n)
            out.append((os.path.join(GEN, "aw_pass_%s_%d.cu" % (tag, n)), text))
    for tag, vt in FORMS:
        text = "// generated by _build.py: grouped %s pass kernels\n" % tag
        text += '#include "aw_group.cuh"\n\nAW_GROUP_LAUNCHER(%s, %s)\n' % (vt, tag)
        out.insert(0, (os.path.join(GEN, "aw_group_%s.cu" % tag), text))
    return out
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
    os.makedirs(GEN, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    units = []
    for path, text in _generated():
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
        units.append(path)
    units += [os.path.join(CSRC, src) for src in SOURCES]
    for s in units:
        o = os.path.join(BUILD, os.path.basename(s).replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + deps):
            jobs.append([_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                            "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    if jobs:
        workers = min(len(jobs), max(2, (os.cpu_count() or 4)))
        with ThreadPoolExecutor(max_workers=workers) as ex:
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
