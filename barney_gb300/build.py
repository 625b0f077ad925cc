"""Builds the native library in-tree: barney_gb300/_lib/libbarney_gb300.so,
and the synthetic-input generator beside it (barney_gb300/_lib/libgbv_scenegen.so,
host code only, kept out of the renderer's library).

Every CUDA translation unit is compiled for sm_103a only, in parallel, with
``-fmad=false`` so no multiply-add is fused (the path reproduces the
reference's FP32 arithmetic operation by operation); host code is compiled
with ``-ffp-contract=off`` for the same reason.
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
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIBNAME = "libbarney_gb300.so"
SCENEGEN = PKG / "scenegen"
SCENEGEN_LIB = "libgbv_scenegen.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def scenegen_path() -> Path:
    return LIBDIR / SCENEGEN_LIB


def build_scenegen(force: bool = False) -> Path:
    """The input generator: one g++ step, no CUDA."""
    LIBDIR.mkdir(parents=True, exist_ok=True)
    out = scenegen_path()
    deps = sorted(SCENEGEN.glob("*.cpp")) + sorted(SCENEGEN.glob("*.h"))
    if force or _stale(out, deps):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", "-Wall",
              *[str(d) for d in deps if d.suffix == ".cpp"], "-o", str(out)])
    return out


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OBJDIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJDIR / (src.stem + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        jobs.append((obj, [src, *headers], cmd))
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJDIR / (src.stem + ".o")
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall",
               "-I", str(INCLUDE), "-I", str(cuda / "include"), "-c", str(src), "-o", str(obj)]
        jobs.append((obj, [src, *headers], cmd))
    todo = [(o, c) for (o, d, c) in jobs if force or _stale(o, d)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(_run, c): o for (o, c) in todo}
        for f in cf.as_completed(futs):
            f.result()
            if verbose:
                print("built", futs[f].name, file=sys.stderr)
    objs = [str(o) for (o, _, _) in jobs]
    out = lib_path()
    if force or not out.exists() or any(Path(o).stat().st_mtime > out.stat().st_mtime for o in objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(out), *objs, "-lpthread"])
    build_scenegen(force)
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
