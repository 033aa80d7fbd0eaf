"""Build recipe for libooc_svo_gpu.so and the svo_builder command lines (in-tree).

Translation units compile in parallel; CUDA code targets sm_103a only and is
compiled with -fmad=false and -ffp-contract=off so that every FP32 operation
rounds once, like the reference's x86-64 build.  IEEE division and square root
are nvcc's defaults and fast-math is never enabled.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libooc_svo_gpu.so")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-v"]
CUDA_SOURCES = ["ooc_kernels.cu", "ooc_api.cu", "ooc_noalloc.cu", "ooc_validate.cu"]
CXX_SOURCES = ["ooc_files.cpp", "ooc_server.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd, log=None):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if log is not None:
        log.append(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (p.returncode, " ".join(cmd), p.stdout))
    return p.stdout


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile the library and the two CLIs; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "ooc_svo_gpu.h"))
    log: list = []
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", cuda_inc,
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(lambda c: _run(c, log), jobs):
            pass
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread"], log)
    main = os.path.join(CSRC, "svo_builder_main.cpp")
    for name, extra in (("svo_builder", []), ("svo_builder_binary", ["-DOOC_CLI_BINARY"])):
        exe = os.path.join(BIN, name)
        if force or not _newer(exe, [main, LIB, os.path.join(INCLUDE, "ooc_svo_gpu.h")]):
            _run(["g++", "-O2", "-std=c++17", *extra, "-I", INCLUDE, main, "-o", exe, "-L", PKG, "-looc_svo_gpu",
                  "-Wl,-rpath,$ORIGIN/.."], log)
    check = os.path.join(CSRC, "octree_check_main.cpp")
    exe = os.path.join(BIN, "octree_check")
    if force or not _newer(exe, [check, LIB, os.path.join(INCLUDE, "ooc_svo_gpu.h")]):
        _run([nvcc, "-O2", "-std=c++17", "-I", INCLUDE, check, "-o", exe, "-L", PKG, "-looc_svo_gpu",
              "-Xlinker", "-rpath,$ORIGIN/.."], log)
    if verbose:
        sys.stdout.write("".join(log))
    return LIB


# Where this build recipe looks for the reference's sources when OOC_REFERENCE is not set:
# the read-only mount of the container the project is developed in.  The sources are only
# compiled into oracle/_ref (test infrastructure); nothing else reads them.
REFERENCE_MOUNT = "/root/reference"


def reference_dir() -> str:
    """Where the reference's sources are read from: OOC_REFERENCE, else REFERENCE_MOUNT."""
    return os.environ.get("OOC_REFERENCE") or REFERENCE_MOUNT


def reference_present() -> bool:
    return os.path.isdir(os.path.join(reference_dir(), "src", "svo_builder"))


def build_reference(target: str = "ref") -> None:
    """Compile the reference's own sources with the oracle recipe (make -C oracle <target>)."""
    _run(["make", "-C", os.path.join(ROOT, "oracle"), target, "REF=" + reference_dir()])


def build_oracle(verbose: bool = False) -> None:
    """Compile the CPU oracle (and the reference build when its sources are present)."""
    oracle = os.path.join(ROOT, "oracle")
    out = _run(["make", "-C", oracle, "all"])
    if reference_present():
        out += _run(["make", "-C", oracle, "ref", "REF=" + reference_dir()])
    if verbose:
        sys.stdout.write(out)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    build_oracle(verbose=True)
