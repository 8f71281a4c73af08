"""Builds libibisgb.so in-tree (ibis_gb300/_build/) for sm_103a.

Host code is compiled without FMA contraction (-ffp-contract=off) so that grid
preprocessing reproduces the reference's geometry bit for bit on both x86 and
aarch64 hosts; kernels_exact.cu is compiled with -fmad=false for the
bitwise-parity FP64 path and kernels_mixed.cu with --use_fast_math (float
division and square root to within 2 ulp, denormals flushed) for the mixed path.  Object files are rebuilt only when a source or
header changes.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libibisgb.so")
DRIVER = os.path.join(OUT, "ibisgb-run")
PYMOD_SRC = os.path.join(SRC, "python", "ibisgb_py.cpp")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp", "-I", SRC, "-I", INCLUDE] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-I", SRC,
             "-I", INCLUDE]

UNITS = {
    "mesh.cpp": "cxx",
    "structured.cpp": "cxx",
    "context.cu": "nvcc",
    "kernels_common.cu": "nvcc",
    "kernels_f64.cu": "nvcc",
    "kernels_mixed.cu": "nvcc-fast",
    "kernels_grad.cu": "nvcc",
    "kernels_ff.cu": "nvcc-fast",
    "kernels_exact.cu": "nvcc-nofma",
    "noalloc.cu": "nvcc",
    "kernels_tangent.cu": "nvcc-nofma",
}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libibisgb")


def _digest(unit: str, flags: list) -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(SRC)):
        if name.endswith((".hpp", ".cuh", ".h")):
            h.update(open(os.path.join(SRC, name), "rb").read())
    h.update(open(os.path.join(INCLUDE, "ibisgb.h"), "rb").read())
    h.update(open(os.path.join(SRC, unit), "rb").read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _compile(unit: str, kind: str, verbose: bool) -> str:
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    if kind == "cxx":
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj]
    else:
        extra = {"nvcc-nofma": ["-fmad=false"], "nvcc-fast": ["--use_fast_math"]}.get(kind, [])
        cmd = [_nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    stamp = obj + ".sha"
    dig = _digest(unit, cmd[1:])
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
        return obj
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {unit} failed:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(dig)
    return obj


def build(verbose: bool = False) -> str:
    """Compile every unit (in parallel) and link libibisgb.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking libibisgb.so failed:\n{r.stdout}\n{r.stderr}")
    # the host driver (ibisgb-run), a client of the C ABI only
    src = os.path.join(SRC, "driver", "ibisgb_run.cpp")
    if not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < max(os.path.getmtime(LIB), os.path.getmtime(src)):
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", INCLUDE, src, "-o", DRIVER,
               "-L", OUT, "-libisgb", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building ibisgb-run failed:\n{r.stdout}\n{r.stderr}")
    build_python_module(verbose)
    return LIB


def python_module_path() -> str:
    import sysconfig
    return os.path.join(HERE, "_ibisgb_py" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_python_module(verbose: bool = False) -> str:
    """The pybind11 module _ibisgb_py (csrc/python/ibisgb_py.cpp), a client of
    libibisgb.so, against the pybind11 headers that ship with torch."""
    import sysconfig
    import torch
    mod = python_module_path()
    inputs = [LIB, PYMOD_SRC, os.path.join(INCLUDE, "ibisgb.h")]
    if os.path.exists(mod) and os.path.getmtime(mod) >= max(os.path.getmtime(p) for p in inputs):
        return mod
    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    py_inc = sysconfig.get_paths()["include"]
    if not os.path.exists(os.path.join(py_inc, "Python.h")):
        print(f"ibis_gb300.build: no Python.h under {py_inc}; _ibisgb_py (torch.autograd bindings) not built",
              file=sys.stderr)
        return ""
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-shared", "-fPIC", "-fvisibility=hidden",
           "-I", INCLUDE, "-I", torch_inc, "-I", py_inc, "-I", os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include"),
           PYMOD_SRC, "-o", mod,
           "-L", OUT, "-libisgb", "-Wl,-rpath,$ORIGIN/_build"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the _ibisgb_py module failed:\n{r.stdout}\n{r.stderr}")
    return mod


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
