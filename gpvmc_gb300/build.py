"""Build the engine's C-ABI shared library in-tree with nvcc for sm_103a.

    python -m gpvmc_gb300.build          # -> gpvmc_gb300/_lib/libgpvmc_gb300.so

Translation units compile in parallel; the link is one nvcc call.  No cmake,
no torch extension machinery: the product is a plain C-ABI .so.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libgpvmc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "model.cpp", "noalloc.cu", "server.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-pthread",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _compile(src, obj, extra):
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + _flags() + extra
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return r.stderr


def build(verbose=False, extra=()):
    """Compile every translation unit and link libgpvmc_gb300.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        logs = list(ex.map(lambda a: _compile(a[0], a[1], list(extra)), zip(SOURCES, objs)))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=[a for a in sys.argv[1:] if a != "-v"]))
