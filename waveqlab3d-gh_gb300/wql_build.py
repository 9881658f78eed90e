"""Build the GB300 library libwql.so in-tree (waveqlab3d-gh_gb300/_build/).

CUDA sources are compiled for sm_103a only, host C++ with g++; translation
units compile in parallel and the library links with a static CUDA runtime,
so the product needs no toolchain at run time.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libwql.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["wql_api.cu", "wql_setup.cu", "wql_volume.cu", "wql_stencil_tma.cu", "wql_interface.cu"]
CPP = ["host/wql_input.cpp", "host/wql_grid.cpp", "host/wql_serve.cpp"]
HEADERS = ["wql_internal.h", "wql_sbp.cuh", "wql_presets.cuh", "wql_stencil.cuh", "host/wql_input.h",
           "host/wql_grid.h", os.path.join("..", "..", "include", "wql.h")]


def _newest(paths):
    return max(os.path.getmtime(os.path.join(CSRC, p)) for p in paths)


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), _newest(HEADERS)):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", "-I" + CSRC, "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-I" + CSRC, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, " ".join(cmd) + "\n" + r.stdout + r.stderr
    return obj, None


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, CU + CPP))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("libwql build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-pthread", "-o", LIB + ".tmp", *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libwql link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
