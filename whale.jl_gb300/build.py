"""Build libwhalegpu.so in-tree (sm_103a only).

Host translation units are compiled with g++, the CUDA one with nvcc
(-gencode arch=compute_103a,code=sm_103a), all in parallel, then linked with
nvcc into ``_build/libwhalegpu.so`` next to this file.  No cmake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwhalegpu.so")
# the host parts alone (model, ALE reader, packer, workload generator,
# tracking; no CUDA): for processes that must not load the GPU library
HOST_LIB = os.path.join(OUT, "libwhalehost.so")

CXX_SRCS = ["wg_api.cpp", "wg_model.cpp", "wg_ccd.cpp", "wg_pack.cpp", "wg_synth.cpp", "wg_track.cpp"]
CU_SRCS = ["wg_kernels.cu", "wg_nowhere.cu", "wg_track_dev.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwhalegpu")
    return p


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, "wg_internal.h"), os.path.join(CSRC, "wg_nowhere.h"), os.path.join(CSRC, "wg_track_dev.h"),
               os.path.join(HERE, "..", "include", "whalegpu.h")]
    nvcc = _nvcc()
    inc = ["-I", os.path.join(_cuda_home(), "include")]
    jobs = []
    objs = []
    for s in CXX_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            # no FMA contraction: host arithmetic rounds the same on x86 and Arm
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", *inc,
                   "-c", src, "-o", obj]
            jobs.append(cmd)
    for s in CU_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                   "-c", src, "-o", obj]
            jobs.append(cmd)
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for cmd in jobs]
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out))
        elif verbose and out.strip():
            sys.stderr.write(out)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libwhalegpu build failed:\n" + msg)
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("libwhalegpu link failed:\n" + r.stdout)
    host_objs = objs[: len(CXX_SRCS)]
    if force or jobs or _stale(HOST_LIB, host_objs):
        cmd = ["g++", "-shared", "-o", HOST_LIB, *host_objs, "-Wl,--no-undefined", "-lpthread"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("libwhalehost link failed:\n" + r.stdout)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
