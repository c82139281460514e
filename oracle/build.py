"""Compile the C oracle (``etm_oracle.c``) into ``oracle/_build/libetm_oracle.so`` with gcc -O3 -fopenmp."""

from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "etm_oracle.c"
OUT = HERE / "_build" / "libetm_oracle.so"


def build(verbose: bool = False, force: bool = False) -> Path | None:
    if not SRC.exists():
        return None
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-o", str(OUT), str(SRC)]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    build(verbose=True, force=True)
