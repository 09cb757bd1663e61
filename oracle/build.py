"""ORACLE build recipe (test infrastructure): compiles the C restatements with
gcc into oracle/_build/liboracle.so.  -ffp-contract=off keeps every multiply
and add separately rounded (gcc would otherwise fuse them on aarch64)."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = [HERE / "dda.c", HERE / "mlp_eval.c"]
LIB = HERE / "_build" / "liboracle.so"
FLAGS = ["-O2", "-std=c11", "-shared", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fno-builtin"]


def build(force: bool = False) -> Path:
    srcs = [s for s in SOURCES if s.exists()]
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in srcs):
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", *FLAGS, "-o", str(tmp), *map(str, srcs), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
