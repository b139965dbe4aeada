"""Build ``libcufinufft.so`` (the C-ABI library) in-tree for sm_103a.

Every translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked with cuFFT into ``lib/libcufinufft.so``.  Objects are
rebuilt only when a source or header is newer than them.

    python -m cufinufft_gb300.build        # or cufinufft_gb300.build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import time

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libcufinufft.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC")
    if cand:
        return cand
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags() -> list:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                   "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, verbose: bool) -> tuple:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [nvcc()] + _flags()
    if os.environ.get("CUFINUFFT_PTXAS_VERBOSE"):
        cmd += ["-Xptxas", "-v"]
    cmd += ["-c", src, "-o", obj]
    t0 = time.time()
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
    return obj, r.returncode, time.time() - t0, " ".join(cmd)


def build(verbose: bool = False, jobs: int | None = None, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hmt = _headers_mtime()
    todo = []
    for s in srcs:
        obj = os.path.join(OBJ, os.path.basename(s) + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(s), hmt):
            todo.append(s)
    jobs = jobs or max(1, os.cpu_count() or 1)
    failed = []
    if todo:
        # longest translation units first keeps the parallel build short
        todo.sort(key=lambda s: ("si_" not in s, "3" not in os.path.basename(s)))
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for obj, rc, dt, cmd in ex.map(lambda s: _compile(s, verbose), todo):
                if verbose:
                    print(f"  {os.path.basename(obj)}: {dt:.1f}s", flush=True)
                if rc != 0:
                    failed.append(cmd)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    objs = [os.path.join(OBJ, os.path.basename(s) + ".o") for s in srcs]
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    t0 = time.time()
    path = build(verbose=True, force="--force" in sys.argv)
    print(f"built {path} in {time.time() - t0:.1f}s")
