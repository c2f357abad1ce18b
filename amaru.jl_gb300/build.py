"""Build libamaru_gpu.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel into amaru.jl_gb300/_build/,
then linked into amaru.jl_gb300/amaru_gpu/libamaru_gpu.so.  Objects are
reused when newer than their source and the shared headers.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "amaru_gpu", "libamaru_gpu.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
SOURCES = ["shapes.cpp", "pattern.cu", "element.cu", "solver.cu", "capi.cu", "batch.cu", "server.cu", "amg.cu", "recovery.cu", "dyn.cu", "modal.cu", "vtu.cpp", "peak.cu", "coupled.cu"]


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".h")]
    hs.append(os.path.join(INCLUDE, "amaru_gpu.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, verbose=False):
    path = os.path.join(SRC, src)
    obj = os.path.join(OUT_DIR, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), _headers()):
        return obj
    # host code without FMA contraction: the shape tables must be bitwise reproducible on x86 and Arm
    cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE,
           "-I", SRC,
           "--expt-relaxed-constexpr", "-c", path, "-o", obj + ".tmp"]
    if src.endswith(".cpp"):
        cmd = [NVCC, "-std=c++17", "-O3", "-x", "cu", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off", "-I",
               INCLUDE, "-I", SRC, "-c", path, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OUT_DIR):
            os.remove(os.path.join(OUT_DIR, f))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(SRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
