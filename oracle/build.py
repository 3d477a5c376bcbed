"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/oracle.c (the CPU restatement of the traversals)
  and oracle/ingest.c (the R-MAT writer and the pruners) into oracle/liboracle.so with
  gcc.  It builds on any host (x86 or Arm).
* ``build_ref()`` compiles the reference's own CPU programs from their sources, where
  they lie in the reference tree, into oracle/_ref/ (git-ignored):
  purn-sssp (src/purn-sssp.cpp), purn-ppr (src/purn-ppr.cpp), convert2binary
  (utils/convert2binary.cpp) and ref-bf (oracle/ref_bf_main.cpp linked with
  src/sssp/base-perk/SSSP.cpp, the reference CPU Bellman-Ford) and ref-push
  (oracle/ref_push_main.cpp linked with src/ppr/w-purn-perk/PPR.cpp, the reference
  CPU forward push).  It needs the
  reference tree, so it only runs where that tree is mounted; the reference's CUDA
  programs are not built here.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("C2G_REFERENCE", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(HERE, "liboracle.so")

REF_TOOLS = ("purn-sssp", "purn-ppr", "convert2binary", "ref-bf", "ref-push")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "ingest.c")]
    if force or _stale(ORACLE_SO, srcs):
        _run(["gcc", "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-fPIC", "-shared", "-pthread", "-ffp-contract=off"]
             + srcs + ["-o", ORACLE_SO + ".tmp", "-lm"])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def reference_present():
    return os.path.isfile(os.path.join(REF_ROOT, "src", "purn-sssp.cpp"))


def build_ref(force=False):
    """Compile the reference CPU tools into oracle/_ref/.  Returns the output dir, or
    None when the reference tree is absent."""
    if not reference_present():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    cuda_inc = "/usr/local/cuda/include"
    cuda_lib = "/usr/local/cuda/lib64"
    jobs = {
        "purn-sssp": (["g++", "-O2", "-std=c++17", "-fopenmp", "-I", REF_ROOT,
                       os.path.join(REF_ROOT, "src", "purn-sssp.cpp")],
                      [os.path.join(REF_ROOT, "src", "purn-sssp.cpp")]),
        "purn-ppr": (["g++", "-O2", "-std=c++17", "-fopenmp", "-I", REF_ROOT,
                      os.path.join(REF_ROOT, "src", "purn-ppr.cpp")],
                     [os.path.join(REF_ROOT, "src", "purn-ppr.cpp")]),
        "convert2binary": (["g++", "-O2", "-std=c++17", "-I", REF_ROOT,
                            os.path.join(REF_ROOT, "utils", "convert2binary.cpp")],
                           [os.path.join(REF_ROOT, "utils", "convert2binary.cpp")]),
        "ref-bf": (["g++", "-O2", "-std=c++17", "-I", REF_ROOT,
                    "-I", os.path.join(REF_ROOT, "src", "sssp", "base-perk"), "-I", cuda_inc,
                    os.path.join(HERE, "ref_bf_main.cpp"),
                    os.path.join(REF_ROOT, "src", "sssp", "base-perk", "SSSP.cpp"),
                    "-L", cuda_lib, "-lcudart", "-lpthread", "-Wl,-rpath," + cuda_lib],
                   [os.path.join(HERE, "ref_bf_main.cpp"),
                    os.path.join(REF_ROOT, "src", "sssp", "base-perk", "SSSP.cpp")]),
        "ref-push": (["g++", "-O2", "-std=c++17", "-I", REF_ROOT,
                      "-I", os.path.join(REF_ROOT, "src", "ppr", "w-purn-perk"), "-I", cuda_inc,
                      os.path.join(HERE, "ref_push_main.cpp"),
                      os.path.join(REF_ROOT, "src", "ppr", "w-purn-perk", "PPR.cpp"),
                      "-L", cuda_lib, "-lcudart", "-lpthread", "-Wl,-rpath," + cuda_lib],
                     [os.path.join(HERE, "ref_push_main.cpp"),
                      os.path.join(REF_ROOT, "src", "ppr", "w-purn-perk", "PPR.cpp")]),
    }
    for name, (cmd, srcs) in jobs.items():
        out = os.path.join(REF_OUT, name)
        if force or _stale(out, srcs):
            _run(cmd + ["-o", out + ".tmp"])
            os.replace(out + ".tmp", out)
    return REF_OUT


def ref_tool(name):
    p = os.path.join(REF_OUT, name)
    return p if os.path.isfile(p) and os.access(p, os.X_OK) else None


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
