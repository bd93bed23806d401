"""Builds the engine's native libraries in-tree.

    lib/libpatchmatch_gb300.so   CUDA engine + C ABI (sm_103a only)
    lib/libpm_scene.so           seeded synthetic scene generator (host C++)
    lib/pm_cli                   command-line driver mirroring the reference's main.cpp

Translation units compile in parallel; each step is skipped when its output is newer than
its inputs. Run: python -m patchmatch_cuda_gb300.build
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
LIB = PKG / "lib"
OBJ = PKG / "_build"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall"]

# window-templated kernels: 4 window groups x 2 samplers x 2 plane modes
WINDOW_SOURCES = [f"pm_win_{g}{hw}{pl}.cu" for pl in ("", "_pl") for hw in ("", "_hw") for g in "dcba"]
CUDA_SOURCES = WINDOW_SOURCES + ["pm_prep.cu", "pm_api.cu", "pm_noalloc.cu", "pm_gemm.cu", "pm_net.cu",
                                 "pm_proposal.cu", "pm_fuse.cu"]
HEADERS = ["pm_device.cuh", "pm_sweep.cuh", "pm_internal.h", "pm_windows.inc"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> dict[str, Path]:
    nvcc = _nvcc()
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    headers = [CSRC / h for h in HEADERS] + [INCLUDE / "patchmatch_gb300.h"]
    jobs = jobs or max(2, min(len(CUDA_SOURCES) + 2, os.cpu_count() or 4))

    objs = []
    steps = []
    for src in CUDA_SOURCES:
        o = OBJ / (Path(src).stem + ".o")
        objs.append(o)
        if _stale(o, [CSRC / src] + headers):
            steps.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(o)])
    scene_so = LIB / "libpm_scene.so"
    if _stale(scene_so, [CSRC / "pm_scene.cpp", CSRC / "pm_scene.h"]):
        steps.append(["g++", *CXX_FLAGS, "-shared", "-o", str(scene_so), str(CSRC / "pm_scene.cpp")])
    with cf.ThreadPoolExecutor(jobs) as ex:
        for f in [ex.submit(_run, s) for s in steps]:
            f.result()
        if verbose:
            for s in steps:
                print(" ".join(s[:3]), "...", s[-1])

    engine = LIB / "libpatchmatch_gb300.so"
    if _stale(engine, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(engine), *map(str, objs)])
    cli = LIB / "pm_cli"
    if _stale(cli, [CSRC / "pm_cli.cpp", engine, scene_so, INCLUDE / "patchmatch_gb300.h"]):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(INCLUDE), "-o", str(cli), str(CSRC / "pm_cli.cpp"),
              f"-L{LIB}", "-lpatchmatch_gb300", f"-Wl,-rpath,{LIB}"])
    return {"engine": engine, "scene": scene_so, "cli": cli}


if __name__ == "__main__":
    out = build(verbose=True)
    for k, v in out.items():
        print(f"{k}: {v}")
    sys.exit(0)
