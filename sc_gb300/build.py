"""Builds the CUDA library of the GPU path in-tree: sc_gb300/_build/libscgpu.so.

nvcc only (no cmake), one -gencode for sm_103a, translation units compiled in
parallel.  --fmad=false keeps the reference's FP64 operation order (no FMA
contraction) so that verdicts stay bit-identical to the reference's.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libscgpu.so")

SOURCES = ["sc_input.cpp", "sc_context.cu", "energy_kernels.cu", "sweep.cu", "noalloc.cu", "surrogate.cu", "wanglandau.cu",
           "fp64_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
         "--expt-relaxed-constexpr", "-diag-suppress", "1444"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the GPU library cannot be built")
    return exe


def _obj(src):
    return os.path.join(OUT, os.path.splitext(src)[0] + ".o")


def _stale(src):
    obj = _obj(src)
    if not os.path.exists(obj):
        return True
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "sc_gb300.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps) or os.path.getmtime(__file__) > t


def _compile(src, verbose):
    cmd = [nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", os.path.join(CSRC, src),
                                                                                "-o", _obj(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    todo = [s for s in SOURCES if force or _stale(s)]
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            for s, log in zip(todo, ex.map(lambda s: _compile(s, verbose), todo)):
                logs[s] = log
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + [_obj(s) for s in SOURCES] + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    for s, log in logs.items():
        if log.strip():
            print(f"== {s}\n{log}")
    print(lib)
