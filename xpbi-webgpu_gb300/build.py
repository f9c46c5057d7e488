"""Build libxpbi.so (the sm_103a CUDA library behind include/xpbi.h) in-tree.

Each translation unit is compiled by its own nvcc process in parallel, then
linked with the static CUDA runtime into ``libxpbi.so`` next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libxpbi.so")
SOURCES = ["api.cu", "api_mlp.cu", "sort.cu", "solve.cu", "mlp.cu", "noalloc.cu", "render.cu", "sample.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libxpbi")
    return exe


def _flags(extra: list[str] | None = None) -> list[str]:
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo",
             "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
             "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if extra:
        flags += extra
    return flags


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_v: bool = False, force: bool = False, out: str | None = None,
          extra: list[str] | None = None, build_dir: str | None = None) -> str:
    """Compile every .cu for sm_103a and link libxpbi.so; returns its path.

    out / build_dir / extra (nvcc flags such as -DXPBI_MINB_PBF=8) build
    a variant of the library elsewhere without touching the default one."""
    lib = out or LIB
    bdir = build_dir or BUILD
    os.makedirs(bdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "xpbi.h"))
    exe = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *headers, __file__]):
            cmd = [exe, *_flags((["-Xptxas", "-v"] if ptxas_v else []) + (extra or [])), "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd: list[str]) -> tuple[list[str], subprocess.CompletedProcess]:
        return cmd, subprocess.run(cmd, capture_output=True, text=True)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_v:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if jobs or not os.path.exists(lib) or _stale(lib, objs):
        tmp = lib + ".tmp"
        cmd = [exe, "-shared", *ARCH, "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_v="-v" in sys.argv, force="-f" in sys.argv))
