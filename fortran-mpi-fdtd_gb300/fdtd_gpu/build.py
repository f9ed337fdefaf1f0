"""Builds libfdtd_gb300.so in-tree (fortran-mpi-fdtd_gb300/lib/) with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library with the CUDA runtime linked statically.
Host arithmetic (coefficient tables) is compiled without fused multiply-adds
so it gives the same values on x86_64 and aarch64 hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libfdtd_gb300.so")
SOURCES = ["fdtd_api.cu", "fdtd_server.cu", "k2d.cu", "k3d.cu", "k3f.cu", "k2f.cu", "k1d.cu", "kdft.cu", "knoalloc.cu", "ktfsf.cu", "kcheck.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _flags(src):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-I", os.path.join(ROOT, "include"), "-I", CSRC, "--expt-relaxed-constexpr"]
    if src.startswith("k"):
        f += ["-Xptxas", "-v"] if os.environ.get("FDTD_PTXAS_VERBOSE") else []
    return f


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "fdtd_gb300.h"))
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s.replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            jobs.append((s, src, obj))

    def run(job):
        s, src, obj = job
        cmd = [nvcc()] + _flags(s) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for s, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed on {s}")
    objs = [os.path.join(OBJ_DIR, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stdout.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
