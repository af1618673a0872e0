"""Build recipe for libselfgpu.so (sm_103a), compiled in-tree into self_gb300/_build/.

Each translation unit is compiled by its own nvcc / g++ process (in parallel), then linked into one
shared library with a C ABI (include/self_gpu.h).  No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libselfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(SRC) if f.endswith(".cpp"))
    return cu, cpp


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "self_gpu.h"))
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler",
              "-ffp-contract=off", "-lineinfo",
              "--expt-relaxed-constexpr", "-DNDEBUG"] + list(extra_flags)
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + common + ["-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([nvcc] + common + ["-x", "cu", "-c", src, "-o", obj] + ARCH)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        return p.stdout + p.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not os.path.exists(LIB):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
