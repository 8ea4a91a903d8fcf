"""Build libpimd_gb300.so (the C-ABI force engine) in-tree with nvcc for sm_103a.

Each translation unit (.cu, and the host-only .cpp) is compiled in parallel, then linked into one shared library at
pimd-f90_gb300/_build/libpimd_gb300.so. Host code is compiled without floating-point
contraction (-ffp-contract=off) so host-side set-up (k-vectors, normal-mode matrices) rounds
the same way on x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpimd_gb300.so")
SOURCES = ["capi.cu", "neighbors.cu", "pot.cu", "ewald.cu", "mixed.cu", "nm.cu", "peak.cu", "noalloc.cu", "spc.cu",
           "md_batch.cu", "adjoint.cu", "ewald_tc.cu", "contracted.cu", "analysis.cu", "state_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
                   "-fPIC,-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(HERE, "..", "include")]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "pimd_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, os.path.splitext(s)[0] + ".o")
        if force or _stale(obj, src):
            jobs.append([nv] + _flags() + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for r, c in zip(res, jobs):
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(c), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
    objs = [os.path.join(OUT, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        link = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
