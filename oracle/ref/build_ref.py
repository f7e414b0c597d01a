"""Recipe for the reference-built checker: compiles the reference's own
sequential sampler sources (c++/src/mcmc/...) with the shims under
oracle/ref/shim and the harness oracle/ref/ref_harness.cc into
oracle/_ref/libammsb_ref.so.

TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie
(AMMSB_REFERENCE_ROOT, else a `reference` checkout beside this repository's
directory) and writes only into oracle/_ref/.  Missing third-party headers (Boost program_options,
circular_buffer, filesystem, iostreams; google sparsehash; tinyxml2) are
replaced by the small shims; OpenMP and MPI are off (the reference's SEQ
build); Float = float (MCMC_SINGLE_PRECISION, the reference default); the
XML reader is left out.  No reference file is modified or copied.
"""
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT, "libammsb_ref.so")
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE_ROOT = os.environ.get("AMMSB_REFERENCE_ROOT",
                                os.path.join(os.path.dirname(REPO), "reference"))
SRC_ROOT = os.path.join(REFERENCE_ROOT, "c++", "src")
SOURCES = ["np", "options", "exception", "random", "data", "network", "timer",
           "preprocess/dataset", "preprocess/relativity", "preprocess/data_factory",
           "learning/learner", "learning/mcmc_sampler_stochastic"]
# headers the reference relied on receiving transitively from older toolchains
FORCE_INCLUDES = ["vector", "limits", "numeric", "climits", "cmath", "cassert"]


def _config(src, dst):
    """config.h from config.h.in: single precision on, everything else off."""
    txt = open(src).read()
    txt = txt.replace("#cmakedefine MCMC_SINGLE_PRECISION", "#define MCMC_SINGLE_PRECISION")
    txt = re.sub(r"#cmakedefine (\w+)", r"/* #undef \1 */", txt)
    os.makedirs(os.path.dirname(dst), exist_ok=True)
    with open(dst, "w") as f:
        f.write(txt)


def available():
    return os.path.isdir(SRC_ROOT)


def build(force=False):
    if not available():
        raise FileNotFoundError("reference sources not found at %s" % SRC_ROOT)
    deps = [os.path.join(HERE, "ref_harness.cc"), os.path.abspath(__file__)]
    for root, _, files in os.walk(os.path.join(HERE, "shim")):
        deps += [os.path.join(root, f) for f in files]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps)):
        return LIB
    gen = os.path.join(OUT, "gen")
    _config(os.path.join(SRC_ROOT, "mcmc", "config.h.in"), os.path.join(gen, "mcmc", "config.h"))
    _config(os.path.join(SRC_ROOT, "dkvstore", "config.h.in"),
            os.path.join(gen, "dkvstore", "config.h"))
    flags = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-DNDEBUG", "-w"]
    for h in FORCE_INCLUDES:
        flags += ["-include", h]
    flags += ["-I" + gen, "-I" + os.path.join(HERE, "shim"), "-I" + SRC_ROOT]
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs = [(os.path.join(SRC_ROOT, "mcmc", s + ".cc"),
             os.path.join(objdir, s.replace("/", "_") + ".o")) for s in SOURCES]
    jobs.append((os.path.join(HERE, "ref_harness.cc"), os.path.join(objdir, "ref_harness.o")))

    def cc(job):
        src, obj = job
        r = subprocess.run(flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("compile %s failed:\n%s" % (src, r.stderr[-4000:]))
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, jobs))
    subprocess.run(["g++", "-shared", "-o", LIB + ".tmp"] + objs, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_if_available():
    """Builds the checker when the reference sources are present (they are
    not on machines that only receive this repository); returns the library
    path or None."""
    if not available():
        return None
    try:
        return build()
    except Exception as e:  # the checker is optional for the product build
        sys.stderr.write("reference checker not built: %s\n" % e)
        return None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
