"""Builds librtcore.so (CUDA kernels + C ABI, sm_103a only) and the rt_sample
drop-in executable in-tree.

    python build-up-phase_gb300/build.py [--force] [--verbose]

Every .cu translation unit is compiled in parallel with

    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false

-fmad=false keeps each float operation separately rounded (FMAs are written
explicitly with __fmaf_rn), which the bit-exact parity with the CPU oracle
depends on.  Outputs: lib/librtcore.so and _build/rt_sample (both ignored by
git; rebuilt on the GPU host, which is aarch64).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
    "--expt-relaxed-constexpr",
    "-I", str(INCLUDE),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librtcore")
    return cand


def lib_path() -> Path:
    return LIB / "librtcore.so"


def sample_path() -> Path:
    return BUILD / "rt_sample"


def _sources() -> list[Path]:
    # kernels (.cu) and host C++ of the library (.cpp); csrc/host/ holds
    # executables, built separately
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        sorted(CSRC.glob("*.cpp")) + sorted((CSRC / "host").glob("*.cpp")) + sorted(INCLUDE.glob("*.h")) + \
        [Path(__file__)]


def _stale(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compiles librtcore.so and rt_sample if any source is newer; returns the
    library path."""
    out = lib_path()
    if not force and not _stale(out) and not _stale(sample_path()):
        return out
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    nv = nvcc()
    flags = NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else [])
    objs = []
    jobs = []
    for src in _sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        jobs.append([nv, *flags, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, verbose or ptxas_info), jobs))
    tmp = out.with_suffix(".so.tmp")
    _run([nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], verbose)
    os.replace(tmp, out)
    sample_src = CSRC / "host" / "rt_sample.cpp"
    if sample_src.exists():
        _run([nv, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I", str(INCLUDE), str(sample_src),
              "-o", str(sample_path()), "-L", str(LIB), "-lrtcore", "-lcudart", f"-Xlinker=-rpath,{LIB}"],
             verbose)
    return out


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print registers / spills per kernel")
    a = ap.parse_args(argv)
    p = build(force=a.force or a.ptxas_info, verbose=a.verbose, ptxas_info=a.ptxas_info)
    print(p)
    return 0


if __name__ == "__main__":
    sys.exit(main())
