"""In-tree build of libgbsp.so (the GB300 path tracer) with nvcc.

    python -m vk_cinematic_gb300.build [--verbose]

Every translation unit is compiled for sm_103a only, in parallel, then
linked into vk_cinematic_gb300/_build/libgbsp.so.  --fmad=false keeps every
a*b+c unfused (the reference's arithmetic rounds after each operation);
kernels that want a fused multiply-add call fmaf explicitly.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgbsp.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["api.cu", "bvh_build.cu", "trace.cu", "pathtrace.cu", "batch.cu", "denoise.cu", "post.cu",
           "compute_pt.cu", "cubemap.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
        "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
    ]


def _deps() -> list[str]:
    out = [os.path.join(INCLUDE, "gbsp.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and not ptxas_info and not _stale(LIB, deps):
        return LIB
    cc = nvcc()
    flags = common_flags() + (["-Xptxas", "-v"] if ptxas_info else [])
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for obj, err in ex.map(compile_one, SOURCES):
            objs.append(obj)
            if verbose or ptxas_info:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.verbose, a.ptxas_info, a.force))
