"""Build script of the in-tree CUDA library 4d_lung_gb300/libcgsense.so.

Compiles every translation unit of csrc/ for sm_103a with nvcc (in
parallel) and links them into one shared library with a plain C ABI
(include/cgsense_c.h).  No CMake: a handful of nvcc invocations.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcgsense.so")
TORCH_LIB = os.path.join(HERE, "libcgsense_torch.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", CSRC, "-I", os.path.join(ROOT, "include")]
FFT_GROUPS = 6


def _units():
    units = []
    for g in range(FFT_GROUPS):
        units.append(("fft_inst.cu", "fft_inst_%d.o" % g, ["-DCGS_FFT_GROUP=%d" % g]))
    for src in ("fft_dispatch.cu", "kernels_misc.cu", "cgs_api.cu", "fft_noalloc.cu", "plain.cu", "fp64.cu", "grad.cu", "io.cu", "spread_csr.cu", "smaps.cu", "toeplitz.cu"):
        units.append((src, src.replace(".cu", ".o"), ["-Xcompiler", "-fopenmp"] if src == "cgs_api.cu" else []))
    units.append(("wave_caipi.cpp", "wave_caipi.o", []))
    units.append(("reco_shim.cpp", "reco_shim.o", []))
    units.append(("voronoi.cpp", "voronoi.o", ["-fopenmp"]))
    return units


def _torch_paths():
    """Include and library directories of the installed PyTorch (libtorch)."""
    import torch
    from torch.utils import cpp_extension
    import io
    import contextlib
    with contextlib.redirect_stderr(io.StringIO()):
        inc = cpp_extension.include_paths()
    return inc, os.path.join(os.path.dirname(torch.__file__), "lib")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "cgsense_c.h"))
    headers.append(os.path.join(ROOT, "include", "cgsense", "Reco.h"))
    cmds = []
    objs = []
    for src, obj, extra in _units():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        if _stale(o, [s, __file__] + headers):
            if src.endswith(".cpp"):
                cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-I", os.path.join(ROOT, "include"),
                       "-I", "/usr/local/cuda/include"] + extra + ["-c", s, "-o", o]
            else:
                cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", s, "-o", o]
            cmds.append(cmd)
    # the libtorch operator (torch_ops.cpp) compiles beside the CUDA units
    tsrc = os.path.join(CSRC, "torch_ops.cpp")
    tobj = os.path.join(BUILD, "torch_ops.o")
    tinc, tlib = _torch_paths()
    if _stale(tobj, [tsrc, __file__, os.path.join(ROOT, "include", "cgsense_c.h")]):
        cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-I", os.path.join(ROOT, "include"),
                     "-I", "/usr/local/cuda/include"] + sum((["-I", d] for d in tinc), []) + ["-c", tsrc, "-o", tobj])
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))

    def run(cmd):
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        return cmd, r.returncode, r.stdout

    if cmds:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for cmd, rc, out in ex.map(run, cmds):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    raise RuntimeError("compilation failed: %s" % cmd[-3])
    if _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + [
            "-cudart", "static", "-lcufft", "-lgomp", "-ldl", "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout)
            raise RuntimeError("link failed")
    if _stale(TORCH_LIB, [tobj, LIB]):
        cmd = ["g++", "-shared", "-o", TORCH_LIB, tobj, "-L", HERE, "-lcgsense", "-L", tlib, "-ltorch", "-ltorch_cpu",
               "-lc10", "-lc10_cuda", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + tlib]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout)
            raise RuntimeError("link of the libtorch operator failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
