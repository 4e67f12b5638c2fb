"""Build recipe of the GB300 library (in-tree, sm_103a only).

Compiles the CUDA translation units and the C++ host builder in parallel and
links ``sem2dpack_gb300/_lib/libsem2d_gb300.so``.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libsem2d_gb300.so")
# objects of this machine's architecture (the host and the GPU machine differ)
OBJ_DIR = os.path.join(OUT_DIR, "obj-" + platform.machine())
CU_SOURCES = ["sem2d_gpu.cu", "bulk_launch.cu", "bulk_n3.cu", "bulk_n5.cu", "bulk_n6.cu", "bulk_n9.cu", "noalloc.cu",
              "adjoint.cu", "march.cu"]
CPP_SOURCES = ["host_builder.cpp", "abi_layout.cpp", "autotune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return files + [os.path.abspath(__file__)]


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile if any source is newer than the library; return the library path."""
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    # an object is rebuilt when its source, a header or this recipe is newer
    headers = [f for f in _deps() if not f.endswith((".cu", ".cpp"))]
    t_headers = max(os.path.getmtime(f) for f in headers)

    def stale(src, obj):
        return force or ptxas_verbose or not os.path.exists(obj) or \
            os.path.getmtime(obj) < max(t_headers, os.path.getmtime(src))

    objs, cmds = [], []
    for src in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        cmd = [nv, "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-lineinfo", "-std=c++17",
               "-Xcompiler", "-fPIC", "-I" + INCLUDE, "--expt-relaxed-constexpr"] + ARCH
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        objs.append(obj)
        if stale(os.path.join(CSRC, src), obj):
            cmds.append(cmd)
    for src in CPP_SOURCES:
        obj = os.path.join(OBJ_DIR, src.replace(".cpp", ".o"))
        if stale(os.path.join(CSRC, src), obj):
            cmds.append(["g++", "-c", os.path.join(CSRC, src), "-o", obj, "-O2", "-std=c++17", "-fPIC",
                         "-ffp-contract=off", "-Wall", "-I" + INCLUDE])
        objs.append(obj)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(cmds)))) as ex:
        outs = list(ex.map(run, cmds))
    if verbose or ptxas_verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp%d" % os.getpid()
    run([nv, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                ptxas_verbose="--ptxas" in sys.argv))
