"""Build the CUDA shared library ``lib/liblbm_gb300.so`` for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and linked into one shared
library whose exported symbols are the C ABI of ``include/lbm_gb300.h``.
The build is skipped when the library is newer than every source and header.

    python -m lbm_jax_autodiff_gb300.build [--force]
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "liblbm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no a*b+c contraction, so host-side constants round the same on
# x86-64 and aarch64 (where GCC would otherwise fuse them)
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = sources()
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_flags=(), lib=None):
    """Compile and link; returns the library path.  ``extra_flags`` (e.g.
    ``-DLBM_ADJ_MINB=2``) and ``lib`` build a variant next to the default."""
    out_lib = lib or LIB
    if not force and not extra_flags and lib is None and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()

    tag = "" if lib is None else "_" + os.path.basename(lib).replace(".so", "")

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + tag + ".o")
        cmd = [nvcc, *NVCC_FLAGS, *extra_flags, *ARCH, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr.strip():
            sys.stderr.write(r.stderr)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out_lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, out_lib)
    return out_lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
