"""Build recipe of the CPU oracle (test infrastructure): oracle/liboracle.so.

gcc, -O2, OpenMP when the compiler has it.  Only tests/, bench.py's CPU
baseline and __graft_entry__.smoke() load the result.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "pmlg_oracle.c"
HDR = HERE / "pmlg_oracle.h"
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    base = [cc, "-O2", "-fPIC", "-shared", "-std=gnu11", str(SRC), "-o", str(LIB) + ".tmp"]
    r = subprocess.run(base[:2] + ["-fopenmp"] + base[2:], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
