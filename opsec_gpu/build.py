"""Build opsec_gpu/libopsec_gpu.so in-tree with nvcc for sm_103a.

Every translation unit in opsec_gpu/csrc is compiled in parallel into
opsec_gpu/_build/ and linked with cuSOLVER (the FP64 eigensolve), cuBLAS and cuFFT (mock fields).  Host code
carries no architecture-specific flags, so the same recipe builds on x86_64
and aarch64 hosts.

    python -m opsec_gpu.build [--verbose] [--ptxas-info]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libopsec_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, verbose=False, ptxas_info=False):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "opsec_gpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc_path(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    if ptxas_info and src.endswith(".cu"):
        cmd.append("-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
    out = res.stdout + res.stderr
    if verbose and out.strip():
        print(out, file=sys.stderr)
    return obj, out


PROGRAMS = ("basis", "klt", "comma", "dot", "estimate", "mockcounts")
PROG_DIR = os.path.join(HERE, "programs")
BIN = os.path.join(HERE, "bin")


def build_programs():
    """The drop-in programs klt / comma / dot / estimate, linked against the library."""
    os.makedirs(BIN, exist_ok=True)
    common = os.path.join(PROG_DIR, "progs.cpp")
    hdrs = [os.path.join(PROG_DIR, "progs.h"), os.path.join(os.path.dirname(HERE), "include", "opsec_gpu.h")]
    cxx = shutil.which("g++") or "g++"
    out = []
    for name in PROGRAMS:
        exe = os.path.join(BIN, name)
        src = os.path.join(PROG_DIR, name + ".cpp")
        deps = [src, common, LIB] + hdrs
        if os.path.exists(exe) and all(os.path.getmtime(exe) >= os.path.getmtime(d) for d in deps):
            out.append(exe)
            continue
        cmd = [cxx, "-O2", "-std=c++17", "-o", exe, src, common, f"-L{HERE}", "-lopsec_gpu",
               "-Wl,-rpath,$ORIGIN/.."]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"building {name} failed:\n{res.stdout}\n{res.stderr}")
        out.append(exe)
    return out


def build(verbose=False, ptxas_info=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_info), srcs))
    objs = [r[0] for r in results]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc_path())), "lib64")
        cmd = [nvcc_path(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, f"-L{cuda_lib}", "-lcusolver", "-lcublas",
               "-lcufft", "-lcudart", f"-Xlinker=-rpath={cuda_lib}"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(LIB + ".tmp", LIB)
    build_programs()
    return LIB, "".join(r[1] for r in results)


if __name__ == "__main__":
    lib, info = build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas-info" in sys.argv)
    if info.strip():
        print(info)
    print(lib)
