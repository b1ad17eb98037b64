"""Build recipe for libfringe_gb300.so (in-tree, sm_103a).

The library is compiled with nvcc from ``fringe_gb300/csrc`` into
``fringe_gb300/libfringe_gb300.so``; translation units compile in parallel.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "libfringe_gb300.so")
OBJDIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",      # host arithmetic as written (the AD2 threshold)
              "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC"]

SOURCES = ["api.cu", "kernels_f32.cu", "kernels_f64.cu", "gram_box.cu", "batch.cu", "serve.cu", "noalloc.cu",
           "nmap.cu", "integrate.cu", "io.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "fringe_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, verbose):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-I", INCLUDE, "-c", path, "-o", obj]
    else:
        cmd = [_nvcc()] + ["-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                           "-x", "c++", "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compiling %s failed:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libfringe_gb300.so."""
    deps = _deps()
    if not force and not _stale(OUT, deps):
        return OUT
    os.makedirs(OBJDIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", OUT + ".tmp"] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
