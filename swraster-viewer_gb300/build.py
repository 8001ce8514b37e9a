"""Builds libswr.so (CUDA kernels for sm_103a + C++ host runtime + C ABI).

Usage: python build.py [--force]. Objects and the library are written next to
the sources (git-ignored). Translation units compile in parallel; a unit is
rebuilt when it or any header is newer than its object.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libswr.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# -fmad=false / -ffp-contract=off: the reference never fuses a multiply
# and an add, and results must match it bit for bit.
NVCC_FLAGS = [ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
             "-I" + os.path.join(CUDA, "include")]


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "swr.h"))
    return hs


def _compile(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), p.stdout, p.stderr))
    return obj, p.stderr


def build(force=False, verbose=False, defines=(), out=None, lib=None):
    """defines: extra -D flags (variants for experiments build into `out`/`lib`)."""
    global OUT, LIB
    if out:
        OUT, LIB = out, lib
    if defines:
        NVCC_FLAGS.extend("-D" + d for d in defines)
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = ["g++", "-shared", "-o", LIB] + objs + ["-L" + os.path.join(CUDA, "lib64"), "-lcudart_static",
                                                    "-ldl", "-lrt", "-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), p.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
