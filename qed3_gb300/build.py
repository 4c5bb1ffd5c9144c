"""Builds the in-tree CUDA library qed3_gb300/libqed3.so for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared object next to this file.  Host code is compiled with
-ffp-contract=off so the lattice tables are bit-identical on x86-64 and
aarch64 hosts.
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
LIB = os.path.join(HERE, "libqed3.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _needs_rebuild() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "qed3.h"))
    deps.append(__file__)
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not _needs_rebuild():
        build_launch_counter()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-I" + os.path.join(HERE, "..", "include")] + ARCH + (extra or [])

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_launch_counter()
    return LIB


LC = os.path.join(HERE, "liblaunchcount.so")


def build_launch_counter() -> str | None:
    """The benchmark's CUPTI launch counter (launchcount.c, not part of
    libqed3); skipped where the CUPTI headers are missing."""
    src = os.path.join(HERE, "launchcount.c")
    if os.path.exists(LC) and os.path.getmtime(LC) > os.path.getmtime(src):
        return LC
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    inc = [os.path.join(cuda, "include"), os.path.join(cuda, "extras", "CUPTI", "include")]
    libdirs = [os.path.join(cuda, "lib64"), os.path.join(cuda, "extras", "CUPTI", "lib64")]
    cmd = ["gcc", "-O2", "-shared", "-fPIC", "-o", LC + ".tmp", src] + ["-I" + i for i in inc] + \
          ["-L" + l for l in libdirs] + ["-lcupti"] + ["-Wl,-rpath," + l for l in libdirs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    os.replace(LC + ".tmp", LC)
    return LC


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
