"""Builds the engine in-tree: lib/libbfs_gb300.so (C ABI, sm_103a kernels) and
bin/bfs_gb300 (the reference-compatible command line driver).

Usage:  python bfs-gpu-sycl_gb300/build.py [--force] [--jobs N]

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); translation units are compiled in
parallel and only rebuilt when a source or header is newer than its object.
"""
import argparse
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libbfs_gb300.so")
CLI = os.path.join(BINDIR, "bfs_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc():
    path = os.path.join(CUDA_HOME, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def headers():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                out.append(os.path.join(d, f))
    return out


def stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def compile_one(src, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and not stale(obj, [src] + headers()):
        return obj, None
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17",
                                 "-Xcompiler", "-fPIC,-O3", "-I", INCLUDE, "-I", CSRC,
                                 "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O3", "-fPIC", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", CSRC,
               "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force=False, jobs=None, verbose=True):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    # objects built on another host architecture are never reused
    stamp = os.path.join(BUILD, "HOST_ARCH")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        force = True
    if force:
        for d in (BUILD,):
            for f in os.listdir(d):
                if f.endswith(".o"):
                    os.unlink(os.path.join(d, f))
        for f in (LIB, CLI):
            if os.path.exists(f):
                os.unlink(f)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: compile_one(s, force), srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("\n".join(errors))
    objs = [o for o, _ in results]
    if force or stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(HOST, "bfs_main.cpp")
    if os.path.exists(cli_src) and (force or stale(CLI, [cli_src, LIB] + headers())):
        cmd = ["g++", "-O3", "-std=c++17", "-Wall", "-I", INCLUDE, cli_src, "-o", CLI,
               "-L", LIBDIR, "-lbfs_gb300", "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(arch + "\n")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    try:
        build(a.force, a.jobs)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
