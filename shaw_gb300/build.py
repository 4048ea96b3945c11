"""Build libshaw_gpu.so (CUDA kernels + C ABI + host setup) and shaw_exe for sm_103a.

Objects and outputs go to shaw_gb300/_build/.  Translation units compile in
parallel; nvcc cross-compiles for sm_103a without a GPU.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libshaw_gpu.so")
EXE = os.path.join(BUILD, "shaw_exe")
POD_EXE = os.path.join(BUILD, "computeThinSVD")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["fom.cu", "fom_sweep.cu", "fom_band.cu", "rom.cu", "rom_tc.cu", "rom_oz.cu", "rom_batch.cu", "pod.cu"]
CPP_SOURCES = ["host.cpp", "driver.cpp", "rom_driver.cpp", "pod_driver.cpp", "yaml_lite.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build shaw_gb300")
    return cand


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "shaw_gpu.h"))
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-fopenmp",
                                   "-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-I", INCLUDE, "-I", CSRC,
                         "-I", cuda_inc, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcublas", "-lcusolver", "-lgomp"])
    for src, exe in (("main.cpp", EXE), ("pod_main.cpp", POD_EXE)):
        obj = os.path.join(BUILD, src + ".o")
        s = os.path.join(CSRC, src)
        if _stale(obj, [s] + headers):
            _run(["g++", "-O3", "-std=c++17", "-I", INCLUDE, "-c", s, "-o", obj])
        if _stale(exe, [obj, LIB]):
            _run(["g++", "-o", exe, obj, "-L", BUILD, "-lshaw_gpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
