"""Builds the in-tree CUDA library ``synaptogenesis_gb300/_build/libsyngen.so``.

Device code targets sm_103a only (``-gencode arch=compute_103a,code=sm_103a``)
and is compiled with ``--fmad=false``: the simulation cycle reproduces the
reference's floating-point operation order exactly, so no multiply-add may be
contracted.  Host code is plain C++17.  Translation units compile in parallel
and are cached by modification time.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsyngen.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ["-std=c++17", "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I" + os.path.join(CUDA, "include")]


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inl"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "syngen.h"))
    return max(os.path.getmtime(h) for h in hs)


def build(force=False, verbose=False):
    """Compile every translation unit for sm_103a and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_mtime()

    def one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if (not force and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr)):
            return obj
        if src.endswith(".cu"):
            cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (src, r.stdout[-4000:], r.stderr[-6000:]))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, _sources()))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = ["g++", "-shared", "-Wl,-soname,libsyngen.so", "-o", LIB] + objs + [
            "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
