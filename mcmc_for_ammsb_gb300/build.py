"""Build recipe of libammsb_gpu.so (in-tree, sm_103a only).

The library holds the CUDA kernels, the C++ host driver and the C ABI of
include/ammsb_gpu.h.  Translation units compile in parallel and link with
nvcc; the CUDA runtime is linked statically so the library only needs the
driver at run time.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libammsb_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-Wall", "-diag-suppress", "177"]
SOURCES = ["ammsb_gpu.cu", "ammsb_batch.cu", "ammsb_host.cpp", "ammsb_noalloc.cu", "ammsb_adjoint.cu"]
# a standalone measurement executable, not part of the library: the
# random-row gather rate (bench.py --gather-roofline), built on demand
PROBE_SRC = "gather_roofline.cu"
PROBE = os.path.join(HERE, "gather_roofline")


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "ammsb_gpu.h"))
    return files + [os.path.abspath(__file__)]


def build(force=False, verbose=False):
    """Compile libammsb_gpu.so if any source is newer; returns its path."""
    deps = _deps()
    if not force and _newer(LIB, deps) and _newer(CLI, deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_cli()
    return LIB


def build_probe(force=False):
    """The gather-rate probe (csrc/gather_roofline.cu), compiled when it is
    missing or older than its source; returns its path."""
    src = os.path.join(CSRC, PROBE_SRC)
    if not force and _newer(PROBE, [src, os.path.abspath(__file__)]):
        return PROBE
    cmd = [_nvcc()] + ARCH + ["-O3", "-std=c++17", src, "-o", PROBE + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (PROBE_SRC, " ".join(cmd), r.stderr))
    os.replace(PROBE + ".tmp", PROBE)
    return PROBE


CLI = os.path.join(HERE, "ammsb_main")


def build_cli():
    """The command-line driver (csrc/ammsb_main.cpp), host C++ linked
    against libammsb_gpu.so (found next to it at run time)."""
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(os.path.dirname(HERE), "include"),
           os.path.join(CSRC, "ammsb_main.cpp"), "-L", HERE, "-lammsb_gpu",
           "-Wl,-rpath,$ORIGIN", "-o", CLI + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
