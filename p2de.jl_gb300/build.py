"""Builds libp2de_gpu.so for sm_103a from p2de.jl_gb300/csrc, in-tree (p2de.jl_gb300/_build).

Translation units compile in parallel; the per-degree stage kernels are separate
units so that a rebuild after a change to one file stays short.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libp2de_gpu.so"
# the benchmark's FP64/FP32 FMA-throughput probe (roofline denominator), kept out of the solver
PROBE_SRC = CSRC / "probe" / "p2de_fma_probe.cu"
PROBE_LIB = BUILD / "libp2de_probe.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "p2de.h"]


def _compile(nvcc: str, src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    # the Line path keeps each a*b+c as two rounded operations, as the FP64 restatement does
    extra = ["-fmad=false"] if src.name == "p2de_line.cu" else []
    cmd = [nvcc, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build_probe(force: bool = False, verbose: bool = False) -> Path:
    """libp2de_probe.so: the benchmark's FMA-throughput probe, one translation unit."""
    if not force and PROBE_LIB.exists() and PROBE_LIB.stat().st_mtime >= PROBE_SRC.stat().st_mtime:
        return PROBE_LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = PROBE_LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *NVCC_FLAGS, "-shared", str(PROBE_SRC), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {PROBE_SRC.name}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        build_probe(force, verbose)
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_probe(force, verbose)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
