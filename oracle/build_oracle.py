"""Build the C++ restatement of the split-step loop (oracle/nlm_cpu.cpp) into oracle/_build/libnlm_cpu.so.

TEST INFRASTRUCTURE ONLY: the library is the timed CPU baseline of bench.py and is checked against
the numpy oracle by tests/test_cpu_port.py; nothing in the product loads it.  Portable flags only
(the same source builds on the x86_64 build host and the aarch64 GPU host).
"""

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nlm_cpu.cpp")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnlm_cpu.so")


def build():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(__file__)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O3", "-fno-math-errno", "-fPIC", "-shared", "-pthread", "-Wall", SRC, "-o", tmp]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("building the CPU restatement failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    """The built library with its argument types set."""
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(build())
    d, i, ll, p = ctypes.c_double, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p
    lib.nlmcpu_chi2pdc_green.restype = i
    lib.nlmcpu_chi2pdc_green.argtypes = [i, i, i, d, d, p, p, p, p, d, d, p, i, p, p]
    lib.nlmcpu_chi2pdc_impulses.restype = i
    lib.nlmcpu_chi2pdc_impulses.argtypes = [i, i, i, d, d, p, p, p, d, d, ll, ll, i, p]
    lib.nlmcpu_gnlse_batch.restype = i
    lib.nlmcpu_gnlse_batch.argtypes = [i, i, d, p, p, p, p, ll, p, i, i, p]
    lib.nlmcpu_gnlse_record.restype = i
    lib.nlmcpu_gnlse_record.argtypes = [i, i, d, p, p, p, p, p, i, i, p, p]
    _lib = lib
    return lib


if __name__ == "__main__":
    print(build())
