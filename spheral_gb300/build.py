"""In-tree build of libsphgpu.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel, then linked into
``spheral_gb300/libsphgpu.so``.  Re-running only recompiles sources newer than
their object files.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsphgpu.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

CUDA_SOURCES = ["sort.cu", "hydro.cu", "hydro32.cu", "crk.cu", "crk32.cu", "gravity.cu", "api.cu", "noalloc.cu"]
HOST_SOURCES = ["table.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host arithmetic (kernel-table build) is identical on x86-64 and aarch64
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-lineinfo", "-I" + CSRC, "-I" + INCLUDE]


def _nvcc():
    p = shutil.which("nvcc")
    if p is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return p


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers() + [os.path.abspath(__file__)]
    jobs = []
    objs = []
    sources = [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    for s in sources + HOST_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            if s.endswith(".cu"):
                cmd = [nvcc] + ARCH + COMMON + ["-c", src, "-o", obj]
            else:
                cmd = [nvcc] + COMMON + ["-x", "c++", "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose:
                print(" ".join(cmd))
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
