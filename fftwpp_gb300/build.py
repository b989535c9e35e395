"""In-tree build of lib_fftwpp.so for sm_103a (GB300).

The library is plain CUDA C++ behind a C ABI: no PyTorch headers, so it
builds in seconds with nvcc alone.  Translation units are compiled in
parallel and linked into ``fftwpp_gb300/lib_fftwpp.so``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib_fftwpp.so")
# (source, object, extra flags): kernels.cu is compiled once per precision so
# the two halves of its template instantiations build in parallel.
UNITS = [("kernels.cu", "kernels_f64.o", ["-DFGB_ONLY_DOUBLE"]),
         ("kernels.cu", "kernels_f32.o", ["-DFGB_ONLY_FLOAT"]),
         ("kernels.cu", "kernels_ff.o", ["-DFGB_ONLY_FF"]),
         ("engine.cu", "engine.o", []),
         ("batch.cu", "batch.o", []),
         ("capi.cu", "capi.o", []),
         ("noalloc.cu", "noalloc.o", [])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
         "-I", os.path.join(os.path.dirname(HERE), "include")]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "lib_fftwpp.so")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src, name, extra in UNITS:
        obj = os.path.join(BUILD, name)
        objs.append(obj)
        cmd = [cc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src),
               "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(r.stdout.decode(errors="replace"))
        raise RuntimeError("link failed: " + " ".join(cmd))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
