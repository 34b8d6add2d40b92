"""Build the sm_103a C-ABI library in tree and the CPU checker libraries.

``build_library()`` compiles every ``csrc/*.cu`` translation unit in
parallel with nvcc for ``sm_103a`` and links ``lib/liblns3d_gb300.so``.
``build_oracle()`` runs ``make`` in ``oracle/`` (test infrastructure: the
restated oracle and, where its translated sources exist, the reference).
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "liblns3d_gb300.so"
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_library(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(ROOT, "_build")
    os.makedirs(objdir, exist_ok=True)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(objdir, src[:-3] + ".o")
        out = _run([nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj])
        if verbose and out.strip():
            sys.stdout.write(out)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(8, len(srcs)))) as ex:
        objs = list(ex.map(compile_one, srcs))
    target = os.path.join(LIBDIR, LIBNAME)
    tmp = target + ".tmp"
    _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, target)
    return target


def build_oracle():
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")])


def build_all(verbose=False):
    build_oracle()
    return build_library(verbose=verbose)


if __name__ == "__main__":
    print(build_all(verbose=True))
