"""Builds the CUDA library libkagayaki_gb300.so in-tree for sm_103a.

CUDA sources are compiled by nvcc (-std=c++20, one -gencode for sm_103a),
host sources by g++ (-std=c++23); both with -ffp-contract=off on the host so
the reference-order FP32 sums round identically on x86 and Arm.  Translation
units compile in parallel and are skipped when their object is newer than the
sources and headers.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkagayaki_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_SOURCES = ["bvh.cu", "scene.cu", "trace.cu", "render.cu", "svgf.cu", "nrc.cu", "brdf.cu"]
CPP_SOURCES = ["capi.cpp", "image_io.cpp", "image_load.cpp", "image_formats.cpp", "jpeg_load.cpp", "obj_load.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "kagayaki.h"))
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False, ptxas_info=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        if force or _stale(obj, src, headers):
            cmd = [nvcc, "-std=c++20", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", INCLUDE, "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        if force or _stale(obj, src, headers):
            jobs.append(["g++", "-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", os.path.join(cuda, "include"), "-I", INCLUDE, "-c", src, "-o", obj])
    logs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(lambda c: _run(c, verbose), jobs))
    objs = [os.path.join(BUILD, f + ".o") for f in CU_SOURCES + CPP_SOURCES]
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs], verbose)
    return "".join(logs)


if __name__ == "__main__":
    out = build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    if out:
        print(out)
    print(LIB)
