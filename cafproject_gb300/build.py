"""Build libcube_gb300.so for sm_103a (nvcc, one -gencode, in-tree).

Each translation unit compiles in parallel; the shared library links cuFFT.
The output lives in cafproject_gb300/_build/ (git-ignored) so the library that
the tests and the benchmark load is the one built from this tree.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcube_gb300.so")
SOURCES = ["cube_api.cu", "cube_state.cu", "cube_update.cu", "cube_pm.cu", "cube_pp.cu", "cube_pk.cu", "cube_io.cu", "cube_ic.cu", "cube_timing.cu",
           "cube_dpm.cu", "cube_batch.cu", "cube_sort.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include")]


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "host", "cube_main.cpp")]
    deps.append(os.path.join(HERE, "..", "include", "cube_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in SOURCES]
    if not force and not _stale(objs):
        if not os.path.exists(DRIVER):
            build_driver()
        return LIB
    cc = nvcc()

    def one(src, obj):
        cmd = [cc] + _flags() + list(extra) + ["-c", os.path.join(SRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(one, SOURCES, objs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER_SRC = os.path.join(HERE, "host", "cube_main.cpp")
DRIVER = os.path.join(OUT, "cube_main")


def build_driver():
    """The compiled driver (host/cube_main.cpp): CUBE's step loop calling the
    library through include/cube_gpu.h, linked against the in-tree .so."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include"), DRIVER_SRC,
           "-L" + OUT, "-lcube_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=(["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])))
