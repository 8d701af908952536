"""In-tree build of the native library ``_build/libbgo.so`` (sm_103a only) and
of the tools library ``_build/libbgo_tools.so`` (synthetic genomes and the
integer-pipe probe used by the benchmark and the tests; include/bgo_tools.h).

Each ``csrc/*.cu`` and ``csrc/tools/*.cu`` file is compiled to an object in
parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3``;
the product objects are linked into libbgo.so with the CUDA runtime linked
statically, the tools objects into libbgo_tools.so, which links libbgo.so.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libbgo.so")
TOOLS_PATH = os.path.join(BUILD_DIR, "libbgo_tools.so")
TOOLS = os.path.join(CSRC, "tools")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _inputs():
    return (sorted(glob.glob(os.path.join(CSRC, "*.cu"))),
            sorted(glob.glob(os.path.join(TOOLS, "*.cu"))),
            sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))))


def up_to_date():
    if not os.path.exists(LIB_PATH) or not os.path.exists(TOOLS_PATH):
        return False
    srcs, tools, hdrs = _inputs()
    t = min(os.path.getmtime(LIB_PATH), os.path.getmtime(TOOLS_PATH))
    return all(os.path.getmtime(f) <= t for f in srcs + tools + hdrs + [os.path.abspath(__file__)])


def build(force=False, verbose=False):
    """Compile and link libbgo.so if any source is newer; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs, tools, _ = _inputs()
    nvcc = _nvcc()
    procs = []
    objs, tool_objs = [], []
    for src in srcs + tools:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        (tool_objs if src in tools else objs).append(obj)
        cmd = [nvcc] + ARCH + FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"{s}:\n{o}" for s, o in failed))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB_PATH)
    tmp = TOOLS_PATH + ".tmp"
    cmd = ([nvcc] + ARCH + ["-shared", "-o", tmp] + tool_objs +
           ["-L", BUILD_DIR, "-lbgo", "-Xlinker", "-rpath,$ORIGIN"])
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, TOOLS_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
