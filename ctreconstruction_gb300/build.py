"""Build libctgb.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

    python -m ctreconstruction_gb300.build

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into ``ctreconstruction_gb300/_build/libctgb.so``.  Rebuilds only what
changed.  Only CUDA, nvcc and a host C++ compiler are needed.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libctgb.so")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src, verbose=False):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src), os.path.getmtime(os.path.abspath(__file__))] +
                     [os.path.getmtime(h) for h in headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    # -ffp-contract=off: host arithmetic (the geometry tables, the dominant-axis
    # choice, whose ties the reference's NumPy breaks without fused
    # multiply-adds) rounds the same on x86-64 and aarch64 hosts.
    cmd = [_nvcc(), "-c", src, "-o", obj, "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", INCLUDE, "-I", CSRC, "-lineinfo"]
    if src.endswith(".cu"):
        cmd += ARCH + ["-Xptxas", "-v" if verbose else "-O3"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
