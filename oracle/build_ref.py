"""Recipe: build the reference's own CUDA-C kernels as a host shared library.

Test infrastructure (the CPU baseline and a cross-check of the oracle), never
part of the product.  Steps:

1. When the reference checkout is present, read ``python/GPUFuncs_pycuda.py``
   with ``ast`` and take the exact string it passes to pycuda's
   ``SourceModule`` (GPUFuncs_pycuda.py:7-1193).  Its ``#include`` lines are
   dropped and ``#include "../ref_shim.h"`` is put in front; the result goes to
   ``oracle/_ref/gfp_kernels.cpp`` (git-ignored, so no reference source enters
   the repository's history).
2. Compile that file with ``oracle/ref_launch.cpp`` into
   ``oracle/_ref/libctref.so`` with g++ and OpenMP.

The checkout's location comes from the ``ref_root`` argument, else the
``CTGB_REFERENCE_ROOT`` environment variable, else a checkout named
``reference`` beside this repository's directory.  Where none names a checkout
(a machine that only received the working tree), step 1 is skipped and an
existing ``gfp_kernels.cpp`` is compiled; with neither a checkout nor that
file, ``build`` raises and says how to point it at the reference.
``build(ref_root)`` returns the library path.

    CTGB_REFERENCE_ROOT=/path/to/CTReconstruction python oracle/build_ref.py
    python oracle/build_ref.py /path/to/CTReconstruction
"""
import ast
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
ENV_REF = "CTGB_REFERENCE_ROOT"


SIBLING_REF = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def reference_root(ref_root=None):
    """The reference checkout named by the argument, CTGB_REFERENCE_ROOT or the
    sibling ``reference`` directory, or None."""
    for root in (ref_root, os.environ.get(ENV_REF), SIBLING_REF):
        if root and os.path.isdir(os.path.join(root, "python")):
            return root
    return None


def extract_kernel_text(ref_root):
    path = os.path.join(ref_root, "python", "GPUFuncs_pycuda.py")
    with open(path) as f:
        tree = ast.parse(f.read())
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "SourceModule":
            return node.args[0].value
    raise RuntimeError("SourceModule(...) string not found in %s" % path)


def write_translation_unit(ref_root):
    text = extract_kernel_text(ref_root)
    body = "\n".join(l for l in text.splitlines() if not l.strip().startswith("#include"))
    os.makedirs(OUT, exist_ok=True)
    dst = os.path.join(OUT, "gfp_kernels.cpp")
    with open(dst, "w") as f:
        f.write('// Generated by oracle/build_ref.py from python/GPUFuncs_pycuda.py (not committed).\n')
        f.write('#include "../ref_shim.h"\n')
        f.write(body)
        f.write("\n")
    return dst


def build(ref_root=None, quiet=True):
    src = os.path.join(OUT, "gfp_kernels.cpp")
    root = reference_root(ref_root)
    if root:
        src = write_translation_unit(root)
    if not os.path.exists(src):
        raise RuntimeError("no reference checkout (pass its path, set %s or place it beside the repository "
                           "as 'reference') and no extracted %s"
                           % (ENV_REF, os.path.relpath(src, os.path.dirname(HERE))))
    lib = os.path.join(OUT, "libctref.so")
    deps = [src, os.path.join(HERE, "ref_launch.cpp"), os.path.join(HERE, "ref_shim.h"), os.path.abspath(__file__)]
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps):
        return lib
    # -ffp-contract=off: the rounding the golden vectors were made with (an
    # x86-64 host, no fused multiply-adds), also on aarch64 hosts.
    cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-w", "-o", lib, src,
           os.path.join(HERE, "ref_launch.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if not quiet:
            sys.stderr.write(r.stderr)
        raise RuntimeError("building oracle/_ref/libctref.so failed:\n" + r.stderr[-4000:])
    return lib


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, quiet=False))
