"""Build the Origami GB300 library in-tree.

    python origami-sort_gb300/build.py [--verbose] [--force]

Compiles every CUDA translation unit under csrc/ for sm_103a only (one
-gencode), in parallel, and links lib/liborigami_gpu.so. The C++ drivers
(bench_sort, bench_sort_phases) are built into bin/. Sources are rebuilt when
any file under csrc/, include/ or drivers/ is newer than the library.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
DRIVERS = os.path.join(PKG, "drivers")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
SO = os.path.join(LIB, "liborigami_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include"), "-I" + CSRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")
    return exe


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    pats = [os.path.join(CSRC, "*"), os.path.join(REPO, "include", "*"), os.path.join(DRIVERS, "*"),
            os.path.abspath(__file__)]
    return [p for pat in pats for p in glob.glob(pat)]


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def up_to_date():
    return os.path.exists(SO) and os.path.getmtime(SO) >= _newest(_deps())


def build(verbose=False, force=False, ptxas_info=False):
    if not force and up_to_date():
        return SO
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nv = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    objs = []
    jobs = []
    for src in _sources():
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        jobs.append([nv, *ARCH, *NVFLAGS, *extra, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        outs = list(ex.map(lambda c: _run(c, verbose), jobs))
    if ptxas_info:
        for o in outs:
            sys.stdout.write(o)
    tmp_so = SO + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp_so, *objs], verbose)
    os.replace(tmp_so, SO)
    # C++ drivers linked against the library and the CUDA runtime
    cuda_home = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    cuda_lib = next((p for p in (os.path.join(cuda_home, "lib64"), os.path.join(cuda_home, "lib"))
                     if os.path.isdir(p)), os.path.join(cuda_home, "lib64"))
    djobs = []
    for drv in sorted(glob.glob(os.path.join(DRIVERS, "*.cpp"))):
        exe = os.path.join(BIN, os.path.basename(drv)[:-4])
        djobs.append(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include"),
                      "-I" + os.path.join(cuda_home, "include"), drv, "-o", exe, "-L" + LIB, "-lorigami_gpu",
                      "-L" + cuda_lib, "-lcudart", "-Wl,-rpath," + LIB, "-Wl,-rpath," + cuda_lib, "-pthread"])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(djobs))) as ex:
        list(ex.map(lambda c: _run(c, verbose), djobs))
    return SO


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print -Xptxas -v register/smem usage")
    a = ap.parse_args()
    print(build(verbose=a.verbose, force=a.force or a.ptxas_info, ptxas_info=a.ptxas_info))
