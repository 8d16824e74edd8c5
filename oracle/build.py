"""Builds the oracle (test infrastructure only): liboracle.so from the C++ restatement of parry3d.

Only tests/, the smoke check and the bench's CPU-baseline leg load it, as the checker. Compiled
with -ffp-contract=off so no multiply-add is fused (Rust never contracts), and without any
-ffast-math style flag, so every f32/f64 operation rounds as IEEE arithmetic in the reference.
No architecture-specific flags: the same source builds on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    srcs = [HERE / "capi.cpp"]
    deps = srcs + list(HERE.glob("*.hpp")) + [Path(__file__)]
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in deps):
        return LIB
    cxx = shutil.which("g++") or "c++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
           "-o", str(tmp)] + [str(s) for s in srcs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
