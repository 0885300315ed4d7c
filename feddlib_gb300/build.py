"""Builds feddlib_gb300/libfeddgpu.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel; `-Xptxas -v` output (registers,
spills, shared memory per kernel) lands in feddlib_gb300/_build/ptxas.log.
Usage:  python -m feddlib_gb300.build   (or __graft_entry__.build()).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfeddgpu.so")
SOURCES = ["graph.cu", "k_hyper.cu", "k_ns.cu", "k_scalar.cu", "k_rhs.cu", "k_bc.cu", "k_gn.cu", "mlp.cu", "capi.cu",
           "mesh.cu", "tables.cpp", "gen.cpp", "medit.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "feddgpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj, ""
    cmd = [nvcc(), "-c", path, "-o", obj, "-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-lineinfo",
           "--expt-relaxed-constexpr"] + ARCH
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "cu"]
    if src == "gen.cpp":
        # no fused multiply-add contraction on any host (aarch64 gcc contracts
        # by default): the device generator in mesh.cu rounds every operation
        # and matches this one bit for bit
        cmd += ["-Xcompiler", "-ffp-contract=off"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, SOURCES))
    with open(os.path.join(BUILD, "ptxas.log"), "a") as f:
        for obj, log in results:
            if log:
                f.write(f"==== {os.path.basename(obj)}\n{log}\n")
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
