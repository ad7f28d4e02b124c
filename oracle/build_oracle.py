"""Compile the C restatement in this folder into ``_build/libhdbscan_oracle.so``.

Test infrastructure: the oracle checks the CUDA path and times the CPU baseline. Plain gcc,
no build system, so the same recipe works on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "hdbscan_oracle.c"
OUTPUT = HERE / "_build" / "libhdbscan_oracle.so"


def build(force: bool = False) -> Path:
    OUTPUT.parent.mkdir(parents=True, exist_ok=True)
    if not force and OUTPUT.exists() and OUTPUT.stat().st_mtime >= SOURCE.stat().st_mtime:
        return OUTPUT
    tmp = OUTPUT.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        os.environ.get("CC", "gcc"), "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-math-errno", "-Wall", "-Wno-unused-function",
        str(SOURCE), "-o", str(tmp), "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUTPUT)
    return OUTPUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
