"""Build libhodlrnd_gb300.so in place with nvcc for sm_103a.

    python -m hodlrnd_gb300.build

Each translation unit under csrc/ is compiled in parallel, then linked into
hodlrnd_gb300/libhodlrnd_gb300.so (git-ignored).  Host code is compiled with
-ffp-contract=off: the tree's split planes and admissibility distances must
round exactly as the reference's scalar code.
"""
import concurrent.futures
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhodlrnd_gb300.so")
SOURCES = ["tree.cpp", "aca.cu", "matvec.cu", "gmres.cu", "engine.cu", "noalloc.cu", "vecio.cpp", "server.cpp",
           "tcgen05.cu", "dtree.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = "-fPIC,-fopenmp,-ffp-contract=off,-O2"


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".hpp", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "hodlrnd.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc(), "-c", path, "-o", out, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", HOST_FLAGS]
    if src.endswith(".cu"):
        cmd = cmd[:2] + ARCH + cmd[2:] + ["-Xptxas", "-O3"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return out


def build(force=False):
    os.makedirs(OBJ, exist_ok=True)
    stamp = os.path.join(OBJ, "machine")
    machine = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read() != machine:
        force = True  # objects from another architecture
    if force:
        for f in os.listdir(OBJ):
            if os.path.isfile(os.path.join(OBJ, f)):
                os.remove(os.path.join(OBJ, f))
        if os.path.exists(LIB):
            os.remove(LIB)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    with open(stamp, "w") as f:
        f.write(machine)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
