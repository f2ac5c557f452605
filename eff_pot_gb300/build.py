"""Build libeffpot.so (sm_103a) in-tree with nvcc, one process per unit."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libeffpot.so")
DRIVER = os.path.join(BUILD, "ep_dft4he3d")
DRIVER_SRC = ["ep_fortran_io.cpp", "ep_dft4he3d.cpp"]
UNITS = ["ep_engine_fp64.cu", "ep_engine_fp32.cu", "ep_engine_dd.cu", "ep_engine_dd_x.cu", "ep_engine_dd_xk0.cu",
         "ep_engine_dd_fft.cu", "ep_engine_dd_march.cu", "ep_common.cu", "ep_api.cu", "ep_noalloc.cu",
         "ep_select_pot.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_lib(nv):
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "lib64")


def _stale(src_files, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_files)


def build(verbose=False, force=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "eff_pot.h"))
    nv = nvcc()
    jobs = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale([src] + headers, obj):
            jobs.append([nv, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if force or jobs or _stale(objs, LIB):
        cmd = [nv, *ARCH, "-shared", "-cudart", "shared", "-Xlinker", "-rpath=" + cuda_lib(nv),
               "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libeffpot.so failed")
    build_driver(force=force or bool(jobs))
    return LIB


def build_driver(force=False):
    """The DFT4He3d driver: host C++ over the C ABI, linked to libeffpot.so."""
    ddir = os.path.join(CSRC, "driver")
    srcs = [os.path.join(ddir, f) for f in DRIVER_SRC]
    deps = srcs + [os.path.join(ddir, h) for h in ("ep_fortran_io.h", "ep_instates.h")]
    deps += [os.path.join(ROOT, "include", "eff_pot.h"), LIB]
    if not (force or _stale(deps, DRIVER)):
        return DRIVER
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"), *srcs, "-o", DRIVER,
           "-pthread", "-L" + BUILD, "-leffpot", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cuda_lib(nvcc())]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("build of the ep_dft4he3d driver failed")
    return DRIVER


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
