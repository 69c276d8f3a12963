"""Build recipe for the reference's own OpenMP CPU path (test infrastructure).

This compiles the synaptogenesis reference C++ sources into
``oracle/_ref/libsyngen.so`` so that tests and the CPU-baseline leg of
``bench.py`` can run the reference itself.  Nothing here is part of the product.

Steps
  1. Stage ``src/{core,libs,mpi,ui}`` of the reference checkout into
     ``oracle/_ref/src`` (build scratch, git-ignored, never committed).
  2. Apply four one-line fixes for non-void functions that fall off their end.
     With ``-O2`` g++ treats those paths as unreachable and the library
     crashes; the fixes do not change any arithmetic:
       * ``src/core/util/tools.cpp:3-13``            ``fSet`` returns its value
       * ``src/core/io/buffer.cpp:203-205,216-219``  ``set_*_dirty`` return the flag
       * ``src/core/util/resources/pointer.h:157``    ``operator!=`` returns
       * ``src/core/util/resources/resource_manager.cpp:178-196`` the non-CUDA
         branch of ``allocate_host_pinned`` falls back to ``allocate_host``.
  3. Compile every ``src/core/**/*.cpp`` (except ``main.cpp``) and
     ``src/libs/**/*.cpp`` with
     ``g++ -std=c++11 -O2 -fopenmp -fPIC -pthread -ffp-contract=off -include stdexcept``
     (``__GUI__``/``__MPI__`` undefined so their stubs compile in), then link
     ``libsyngen.so``.

The reference checkout is read from ``$SYNGEN_REFERENCE`` (default: a
``reference`` folder beside this repository's).  When it is absent but a staged copy already exists in
``oracle/_ref/src`` (a machine that received the build folder but not the
checkout), the staged copy is compiled.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
STAGE = os.path.join(REF_DIR, "src")
OBJ = os.path.join(REF_DIR, "obj")
LIB = os.path.join(REF_DIR, "libsyngen.so")

PATCHES = [
    ("core/util/tools.cpp",
     "            if (dist(generator) < fraction) arr[i] = val;\n    }\n}",
     "            if (dist(generator) < fraction) arr[i] = val;\n    }\n    return val;\n}"),
    ("core/io/buffer.cpp",
     "    input_dirty_map[layer] = dirty;\n}",
     "    input_dirty_map[layer] = dirty;\n    return dirty;\n}"),
    ("core/io/buffer.cpp",
     "    auxiliary_dirty_map[layer][key] = dirty;\n}",
     "    auxiliary_dirty_map[layer][key] = dirty;\n    return dirty;\n}"),
    ("core/util/resources/pointer.h",
     "const { !(*this == other); }",
     "const { return !(*this == other); }"),
    ("core/util/resources/resource_manager.cpp",
     "    return ptr;\n#endif\n}\n\nvoid* ResourceManager::allocate_device",
     "    return ptr;\n#else\n    return allocate_host(count, size);\n#endif\n}\n\n"
     "void* ResourceManager::allocate_device"),
]

CXXFLAGS = ["-std=c++11", "-O2", "-fopenmp", "-fPIC", "-pthread", "-w",
            "-ffp-contract=off", "-include", "stdexcept"]


def reference_root():
    """The reference checkout: $SYNGEN_REFERENCE, else a ``reference`` folder
    beside this repository's."""
    repo = os.path.dirname(HERE)
    return os.environ.get("SYNGEN_REFERENCE",
                          os.path.join(os.path.dirname(repo), "reference"))


def stage():
    """Copy the reference sources into the build folder and apply the fixes."""
    src_root = os.path.join(reference_root(), "src")
    if os.path.isdir(STAGE):
        shutil.rmtree(STAGE)
    os.makedirs(REF_DIR, exist_ok=True)
    for sub in ("core", "libs", "mpi", "ui"):
        shutil.copytree(os.path.join(src_root, sub), os.path.join(STAGE, sub))
    for rel, old, new in PATCHES:
        path = os.path.join(STAGE, rel)
        with open(path) as f:
            text = f.read()
        if text.count(old) != 1:
            raise RuntimeError("patch site not found exactly once in " + rel)
        with open(path, "w") as f:
            f.write(text.replace(old, new))


def _sources():
    out = []
    for sub in ("core", "libs"):
        for dirpath, _, files in os.walk(os.path.join(STAGE, sub)):
            for fn in sorted(files):
                if fn.endswith(".cpp") and fn != "main.cpp":
                    out.append(os.path.join(dirpath, fn))
    return sorted(out)


def compile_staged(jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I" + os.path.join(STAGE, d) for d in ("core", "ui", "libs", "mpi")]
    srcs = _sources()

    def one(src):
        obj = os.path.join(OBJ, os.path.relpath(src, STAGE).replace(os.sep, "_") + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
            return obj
        cmd = ["g++"] + CXXFLAGS + inc + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference compile failed: %s\n%s" % (src, r.stderr[-2000:]))
        return obj

    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count()) as ex:
        objs = list(ex.map(one, srcs))
    cmd = ["g++", "-shared", "-fopenmp", "-pthread", "-Wl,-soname,libsyngen.so", "-o", LIB] + objs
    subprocess.run(cmd, check=True)
    return LIB


def build(force=False):
    """Build ``oracle/_ref/libsyngen.so``; returns its path or None if impossible."""
    if os.path.exists(LIB) and not force:
        return LIB
    if os.path.isdir(os.path.join(reference_root(), "src")):
        stage()
    elif not os.path.isdir(STAGE):
        return None
    return compile_staged()


if __name__ == "__main__":
    path = build(force="--force" in sys.argv)
    print(path if path else "reference sources unavailable")
