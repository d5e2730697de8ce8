"""Builds the native library glisser_gb300/_build/libglisser_gb300.so in-tree.

Every CUDA translation unit is compiled for sm_103a only (GB300); host
translation units with g++.  Units compile in parallel and are skipped when
their object is newer than the sources they depend on.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.environ.get("GLISSER_BUILD_DIR") or os.path.join(HERE, "_build")
EXTRA_NVCC = os.environ.get("GLISSER_NVCC_FLAGS", "").split()
LIB = os.path.join(OUT, "libglisser_gb300.so")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path())))


def _deps():
    hdrs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hdrs.append(os.path.join(ROOT, "include", "glisser.h"))
    return max(os.path.getmtime(h) for h in hdrs)


# Translation units that must not contract a*b+c into FMA: the device
# interpolation of the planetary history, the device track writer and the
# device planet integrator evaluate the host restatement's formulas in its
# operation order and are compared with it.
PER_FILE_FLAGS = {"interp.cu": ("--fmad=false",), "track.cu": ("--fmad=false",),
                  "planets_dev.cu": ("--fmad=false",)}


def _compile(src, extra_flags=()):
    extra_flags = tuple(extra_flags) + PER_FILE_FLAGS.get(os.path.basename(src), ())
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps()):
        return obj
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc_path(), GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-Xptxas", "-warn-spills", *inc, *EXTRA_NVCC, *extra_flags, "-c", src, "-o", obj + ".tmp"]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
               "-I" + os.path.join(cuda_home(), "include"), *inc, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as pool:
        objs = list(pool.map(_compile, srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc_path(), GENCODE, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    build_cli()
    if verbose:
        print("built", LIB)
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "glisser_main.cpp")
CLI = os.path.join(OUT, "glisser")


def build_cli():
    """The glisser command (cli/glisser_main.cpp) linked against the library,
    which it finds next to itself."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(LIB)):
        return CLI
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"), CLI_SRC, "-o", tmp,
           "-L" + OUT, "-lglisser_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("glisser command build failed: %s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
