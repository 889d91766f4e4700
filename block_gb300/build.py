"""Build of the native library (host C++ + sm_103a CUDA) into
block_gb300/_build/libblockgb300.so.  No cmake; sources compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libblockgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    host = sorted(os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host")) if f.endswith(".cpp"))
    cuda = sorted(os.path.join(CSRC, "cuda", f) for f in os.listdir(os.path.join(CSRC, "cuda")) if f.endswith(".cu"))
    cuda.append(os.path.join(CSRC, "capi.cu"))
    return host, cuda


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stderr


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    host, cuda = _sources()
    objs, cmds = [], []
    for s in host:
        o = os.path.join(OUT, "h_" + os.path.basename(s) + ".o")
        cmds.append(["g++", "-std=c++17", "-O3", "-fPIC", "-Wall", "-c", s, "-o", o])
        objs.append(o)
    for s in cuda:
        o = os.path.join(OUT, "c_" + os.path.basename(s) + ".o")
        cmds.append([nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-c", s, "-o", o])
        objs.append(o)
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        for l in logs:
            if l.strip():
                print(l, file=sys.stderr)
    tmp = LIB + ".tmp"
    libdir = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xlinker", "-rpath", "-Xlinker", libdir])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
