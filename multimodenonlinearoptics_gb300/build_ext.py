"""Build the engine library ``libnlm_gb300.so`` in-tree.

The CUDA translation units are compiled for sm_103a only, in parallel, with nvcc; the host
engine is compiled with g++; everything is linked into one shared library next to this
file.  Objects are rebuilt only when a source or header is newer than the object.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libnlm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["prop_linear.cu", "prop_direct_a.cu", "prop_direct_b.cu", "prop_gnlse.cu", "kernels_misc.cu",
                "nlm_noalloc.cu", "adjoint.cu", "prop_ragged.cu", "adjoint_gnlse.cu", "prop_ff.cu", "prop_direct_c.cu", "prop_cluster.cu", "prop_cluster_b.cu", "prop_cluster_gnlse.cu", "prop_cluster_pump.cu", "prop_spread.cu", "prop_spread_b.cu",
                "adjoint_gnlse_cluster.cu", "adjoint_cluster.cu", "adjoint_spread.cu",
                "greens_quadrature.cu", "prop_gen_a.cu", "prop_gen_b.cu",
                "prop_gen_c.cu", "prop_gen_d.cu", "prop_gen_e.cu", "prop_spread_fused.cu",
                "prop_spread_w16.cu", "prop_gnlse_spread.cu",
                "adjoint_gnlse_spread.cu", "prop_chi3_pipe.cu"]
CXX_SOURCES = ["engine.cpp", "engine_ragged.cpp"]


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers + [__file__])


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def build(verbose=False, jobs=None):
    """Compile and link the engine library; returns its path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    steps = []
    objs = []
    sources = [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    for src in sources:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, os.path.join(CSRC, src), headers):
            steps.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                          "-I" + INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, os.path.join(CSRC, src), headers):
            steps.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
                          "-I" + os.path.join(cuda, "include"), "-I" + INCLUDE, "-c", os.path.join(CSRC, src),
                          "-o", obj])
    jobs = jobs or max(1, min(len(steps), os.cpu_count() or 1))
    if steps:
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as pool:
            logs = list(pool.map(_run, steps))
        if verbose:
            for cmd, log in zip(steps, logs):
                print(os.path.basename(cmd[-1]), log, file=sys.stderr)
    if steps or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        _run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fPIC"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
