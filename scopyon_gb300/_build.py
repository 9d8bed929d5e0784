"""Build the CUDA library in-tree: ``scopyon_gb300/libscopyon_gb300.so``.

Each ``csrc/*.cu`` file is compiled for sm_103a in parallel into
``scopyon_gb300/_build/`` and the objects are linked into one shared library.
Sources newer than their object are recompiled; nothing else is.

``build_checked()`` builds the same sources with ``-DSC_BOUNDS_CHECK`` into
``scopyon_gb300/_build/checked/libscopyon_gb300_checked.so``: kernels then
range-check their data-dependent shared-memory, tile-buffer and bin-list
indices, skip an access out of range and report it in the status words.
Load it instead of the normal library with ``SCOPYON_GB300_LIB``.
"""

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libscopyon_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def _deps(src):
    deps = [src, os.path.join(INCLUDE, "scopyon_gb300.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    return deps


CHECKED_DIR = os.path.join(BUILD, "checked")
CHECKED_LIB = os.path.join(CHECKED_DIR, "libscopyon_gb300_checked.so")


def _compile(src, extra, out_dir=BUILD):
    obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-I", INCLUDE, "-c", src, "-o", obj]
    # the object is current when it is newer than its sources and was built
    # with the same command line (extra flags rebuild it)
    stamp = obj + ".cmd"
    line = " ".join(cmd)
    same_cmd = os.path.exists(stamp) and open(stamp).read() == line
    if (same_cmd and os.path.exists(obj) and
            all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in _deps(src))):
        return obj, None
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        return obj, "%s\n%s%s" % (line, proc.stdout, proc.stderr)
    with open(stamp, "w") as f:
        f.write(line)
    return obj, None


def build(verbose=False, extra_flags=(), out_dir=BUILD, lib=LIB):
    """Compile and link the library; return its path."""
    os.makedirs(out_dir, exist_ok=True)
    sources = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(sources))) as pool:
        results = list(pool.map(lambda s: _compile(s, list(extra_flags), out_dir), sources))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    if verbose:
        print("built", lib)
    return lib


def build_checked(verbose=False):
    """The bounds-checked library (``-DSC_BOUNDS_CHECK``); return its path."""
    return build(verbose, ("-DSC_BOUNDS_CHECK",), CHECKED_DIR, CHECKED_LIB)


if __name__ == "__main__":
    build(verbose=True)
