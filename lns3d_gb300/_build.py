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
PROBE_NAME = "liblns3d_probe.so"
DRIVER_NAME = "lns3d_gpu"
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

    # an object newer than its source, every header and these flags is reused
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps.append(os.path.abspath(__file__))
    newest_dep = max(os.path.getmtime(d) for d in deps)

    def compile_one(src):
        obj = os.path.join(objdir, src[:-3] + ".o")
        srcp = os.path.join(CSRC, src)
        if os.path.exists(obj) and os.path.getmtime(obj) > max(newest_dep, os.path.getmtime(srcp)):
            return obj
        out = _run([nvcc] + NVCC_FLAGS + ["-c", srcp, "-o", obj])
        if verbose and out.strip():
            sys.stdout.write(out)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(8, len(srcs) + 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
        probe = ex.submit(build_probe)
        target = os.path.join(LIBDIR, LIBNAME)
        tmp = target + ".tmp"
        _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, target)
        driver = ex.submit(build_driver)
        probe.result()
        driver.result()
    return target


def build_driver():
    """The host program lns3d_gpu (csrc/host/lns3d_gpu.cpp): the reference's
    implicit run over the C ABI, linked to the library beside it."""
    out = os.path.join(LIBDIR, DRIVER_NAME)
    _run([_nvcc(), "-O2", "-std=c++17", "-o", out + ".tmp", os.path.join(CSRC, "host", "lns3d_gpu.cpp"),
          "-L" + LIBDIR, "-llns3d_gb300", "-Xlinker", "-rpath,$ORIGIN"])
    os.replace(out + ".tmp", out)
    return out


def build_probe():
    """The benchmark's FP64 peak probe, outside the product library."""
    out = os.path.join(LIBDIR, PROBE_NAME)
    _run([_nvcc()] + NVCC_FLAGS + ["-shared", "-o", out + ".tmp", os.path.join(CSRC, "bench", "fp64_probe.cu")])
    os.replace(out + ".tmp", out)
    return out


def build_oracle(refsrc=None):
    """The checker libraries; with refsrc (the reference's src/ directory)
    the reference's own sources are translated under oracle/_ref first."""
    cmd = ["make", "-s", "-j4", "-C", os.path.join(ROOT, "oracle")]
    if refsrc:
        cmd.append("REFSRC=" + refsrc)
    _run(cmd)


def build_all(verbose=False, refsrc=None):
    build_oracle(refsrc)
    return build_library(verbose=verbose)


if __name__ == "__main__":
    print(build_all(verbose=True))
