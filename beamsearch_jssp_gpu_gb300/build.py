"""Build the native library ``_lib/libbsj.so`` (CUDA kernels for sm_103a + C ABI + the
C++ drop-in entry points) with nvcc, in-tree.

Translation units are compiled in parallel and linked into one shared library with the
CUDA runtime linked statically, so the library needs only the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libbsj.so")
OBJ_DIR = os.path.join(OUT_DIR, "_build")
SOURCES = ["bsj_kernels.cu", "bsj_engine.cu", "bsj_compat.cpp", "bsj_noalloc.cu", "bsj_instance.cpp",
           "bsj_server.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbsj.so")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    inc = os.path.join(os.path.dirname(HERE), "include")
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (if stale) and return the path of libbsj.so."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [cc] + ARCH + FLAGS + ["-c", s, "-o", o]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"] if verbose else []
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link of libbsj.so failed")
        os.replace(tmp, LIB)
    build_cli(force=force)
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "bsj_cli.cpp")
CLI_BIN = os.path.join(OUT_DIR, "bsj_cli")
# names the reference's Makefile gives its drivers (Makefile:55-95); each is a link to bsj_cli
CLI_NAMES = ["exec_gpu_v1", "exec_gpu_v2", "exec_gpu_v1_bench", "exec_gpu_v2_bench", "BS-ICH", "BS-PMS",
             "BS-PMS-bench", "exec_cpu_time_width", "exec_time_width"]


def build_cli(force: bool = False) -> str:
    """Compile the command-line drivers against libbsj.so (host C++ only) and link the
    reference's driver names to them in _lib/."""
    inc = os.path.join(os.path.dirname(HERE), "include")
    if force or _stale(CLI_BIN, [CLI_SRC, LIB] + [os.path.join(inc, h) for h in os.listdir(inc)]):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        tmp = CLI_BIN + ".tmp"
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", CLI_SRC, "-o", tmp, "-L" + OUT_DIR, "-lbsj",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("build of bsj_cli failed")
        os.replace(tmp, CLI_BIN)
    for name in CLI_NAMES:
        link = os.path.join(OUT_DIR, name)
        if not os.path.islink(link):
            if os.path.exists(link):
                os.remove(link)
            os.symlink("bsj_cli", link)
    return CLI_BIN


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
