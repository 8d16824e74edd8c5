"""Builds libparrygpu.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

Each .cu translation unit is compiled in parallel, then linked into one shared library next to this
file. Parity-critical code is compiled with --fmad=false (no fused multiply-add contraction), so
the kernels round exactly like the reference's f32 arithmetic; translation units listed in
FMAD_OK (tensor-core MLP code, which has no reference counterpart) keep contraction on.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libparrygpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FMAD_OK = {"mlp.cu"}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libparrygpu")
    return cand


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "parry_gpu.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles and links libparrygpu.so; returns its path. No-op when up to date."""
    if not force and not _needs_build():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
                     "-I", str(PKG.parent / "include")]

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        fmad = "--fmad=true" if src.name in FMAD_OK else "--fmad=false"
        cmd = [cc, "-c", str(src), "-o", str(obj), fmad] + common
        if src.suffix == ".cpp":  # host-only code: no contraction of f32 arithmetic (aarch64 gcc contracts by default)
            cmd += ["-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
