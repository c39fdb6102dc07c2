"""Compile the reference's own CUDA-C kernel templates for the CPU.

TEST INFRASTRUCTURE ONLY: used to generate the golden vectors under
``tests/golden/`` (tests/golden/make_golden.py).  ``__graft_entry__.build()``
compiles the modules of the golden configurations where the reference checkout
exists (the build container only); nothing in the library, the GPU tests,
smoke() or bench.py runs them.

The reference keeps its kernels as CUDA-C strings inside Python 2 classes
(e.g. wigner_moyal_cuda_1d.py:624-828) and formats them with str.format
before handing them to PyCUDA's SourceModule.  This module reads those strings
from the reference files as text (the Python 2 modules are not imported),
formats them with the same arguments, prepends the shim in oracle/ref_shim/
(std::complex for pycuda::complex, global thread indices) and compiles each
module with g++ into oracle/_ref/.  A generated launcher per kernel loops over
the launch grid on the CPU.  cuFFT is not part of these modules; the harness
(oracle/ref_kernels.py) supplies NumPy FFTs in its place.
"""
import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $AW_REFERENCE_DIR, else a folder named "reference" beside this repository
REF = os.environ.get("AW_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")

_GLOBAL = re.compile(r"__global__\s+void\s+(\w+)\s*\(([^)]*)\)")


def available():
    return os.path.isdir(REF)


def template(filename, name):
    """The text of the class attribute `name = \"\"\"...\"\"\"` in a reference file."""
    text = open(os.path.join(REF, filename)).read()
    m = re.search(r"^[ \t]*%s\s*=\s*\"\"\"(.*?)\"\"\"" % re.escape(name), text, re.S | re.M)
    if not m:
        raise KeyError("%s not found in %s" % (name, filename))
    return m.group(1)


def _params(plist):
    out = []
    for p in plist.split(","):
        p = p.strip()
        if not p:
            continue
        m = re.match(r"(.*?)(\w+)$", p)
        ctype, pname = m.group(1).strip(), m.group(2)
        out.append((ctype, pname))
    return out


class RefModule:
    """One compiled module; call(kernel, grid, block, *args) runs it on the CPU."""

    def __init__(self, source):
        os.makedirs(OUT, exist_ok=True)
        kernels = _GLOBAL.findall(source)
        launchers = ["aw_ref_dim3 blockIdx, threadIdx, blockDim;"]
        self.sigs = {}
        for name, plist in kernels:
            params = _params(plist)
            self.sigs[name] = params
            decl = ", ".join("%s %s" % (t, n) for t, n in params)
            call = ", ".join(n for _, n in params)
            launchers.append(
                'extern "C" void aw_ref_launch_%s(int gx, int gy, int bx%s) {\n'
                "  blockDim.x = bx; blockDim.y = 1; blockDim.z = 1;\n"
                "  for (int by_ = 0; by_ < gy; ++by_)\n"
                "    for (int bx_ = 0; bx_ < gx; ++bx_)\n"
                "      for (int tx_ = 0; tx_ < bx; ++tx_) {\n"
                "        blockIdx.x = bx_; blockIdx.y = by_; blockIdx.z = 0;\n"
                "        threadIdx.x = tx_; threadIdx.y = 0; threadIdx.z = 0;\n"
                "        %s(%s);\n"
                "      }\n}\n" % (name, (", " + decl) if decl else "", name, call))
        # some templates (the fill kernels) include only math.h; the shim supplies the thread indices
        full = "#include <pycuda-complex.hpp>\n" + source + "\n" + "\n".join(launchers)
        key = hashlib.sha1(full.encode()).hexdigest()[:16]
        cpp = os.path.join(OUT, "ref_%s.cpp" % key)
        so = os.path.join(OUT, "ref_%s.so" % key)
        if not os.path.exists(so):
            with open(cpp, "w") as fh:
                fh.write(full)
            cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fcx-limited-range", "-ffp-contract=off",
                   "-I" + SHIM, cpp, "-o", so]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            if r.returncode:
                raise RuntimeError("g++ failed on a reference module:\n" + r.stdout)
        self.lib = ctypes.CDLL(so)

    def call(self, name, grid, block, *args):
        fn = getattr(self.lib, "aw_ref_launch_" + name)
        cargs = [ctypes.c_int(grid[0]), ctypes.c_int(grid[1]), ctypes.c_int(block)]
        for (ctype, _), a in zip(self.sigs[name], args):
            if "*" in ctype:
                assert isinstance(a, np.ndarray) and a.flags.c_contiguous
                cargs.append(ctypes.c_void_p(a.ctypes.data))
            elif ctype in ("double", "const double"):
                cargs.append(ctypes.c_double(float(a)))
            else:
                cargs.append(ctypes.c_int(int(a)))
        fn(*cargs)
