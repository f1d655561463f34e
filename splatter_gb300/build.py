"""Builds libsplatter_cuda.so in-tree (splatter_gb300/_build/) with nvcc for sm_103a.

Every translation unit is compiled with -fmad=false (FP32 results follow the written operation
order; fused multiply-adds only where the source says fmaf) and IEEE division/sqrt (nvcc's
defaults).  Host code is compiled with -ffp-contract=off for the same reason.  The CUDA runtime is
linked as a shared library so the library shares one runtime with PyTorch when both are loaded.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsplatter_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "splatter.h"))
    return hs


def _flags():
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
            "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", "-I", CSRC,
            "-I", os.path.join(ROOT, "include")]


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    newest_hdr = max(os.path.getmtime(h) for h in _headers())
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            cmd = [nvcc, *_flags(), "-c", s, "-o", o]
            if s.endswith(".cpp"):
                cmd = [nvcc, *_flags(), "-x", "cu", "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        return p.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", LIB + ".tmp", *objs,
               "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        run(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
