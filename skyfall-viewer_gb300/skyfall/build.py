"""In-tree build of the skyfall CUDA library (libskyfall.so).

Compiles every translation unit under ../csrc for sm_103a with nvcc, in
parallel, and links them into skyfall/libskyfall.so next to this file.
Objects go to ../_build/.  No cmake, no torch: plain nvcc.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                      # skyfall-viewer_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIB = PKG_DIR / "libskyfall.so"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    # IEEE f32 in source order: no contraction into FMA (the few deliberate
    # fused multiply-adds are written as __fmaf_rn).
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    objs = []
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        p = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, p

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            for src, cmd, p in ex.map(run, jobs):
                if verbose or ptxas_info:
                    sys.stderr.write(p.stdout + p.stderr)
                if p.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{p.stdout}{p.stderr}")
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{p.stdout}{p.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
