"""Build recipe for the C^2graph GB300 library (no cmake).

Compiles every translation unit in csrc/ in parallel (nvcc for .cu with
``-gencode arch=compute_103a,code=sm_103a``, g++ for host .cpp), links
lib/libc2graph.so, then the drop-in programs in bin/ (one binary, one symlink per
reference program name).  Outputs stay in-tree and are git-ignored.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OBJ = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(PKG, "lib", "libc2graph.so")
BIN = os.path.join(PKG, "bin")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
             "-I", os.path.join(CUDA_HOME, "include")]
PROGRAMS = ("sssp-base", "sssp-purn", "ppr-base", "ppr-purn", "adsorption-base", "purn-sssp",
            "purn-ppr", "convert2binary")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(PKG), "include", "c2graph.h"))
    return hs


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _compile(src, hdrs, force):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if force or _newer(obj, [src] + hdrs):
        if src.endswith(".cu"):
            cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj + ".tmp"]
        _run(cmd)
        os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, jobs=None, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    hdrs = _headers()
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdrs, force), srcs))
    if force or _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs +
             ["-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"])
        os.replace(LIB + ".tmp", LIB)
    exe = os.path.join(BIN, "c2g-drop-in")
    cli_src = os.path.join(CLI, "drop_in.cpp")
    if force or _newer(exe, [cli_src, LIB] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-Wall", cli_src, "-o", exe + ".tmp",
              "-L", os.path.dirname(LIB), "-lc2graph", "-Wl,-rpath,$ORIGIN/../lib"])
        os.replace(exe + ".tmp", exe)
    for name in PROGRAMS:
        link = os.path.join(BIN, name)
        if not os.path.islink(link):
            if os.path.exists(link):
                os.remove(link)
            os.symlink("c2g-drop-in", link)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="-f" in sys.argv, verbose=True)
