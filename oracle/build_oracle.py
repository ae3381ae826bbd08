"""Builds the oracle's C part (oracle/c/orc.c) into oracle/_build/liborc.so with gcc -O3
-fopenmp.  Test infrastructure: called by the tests, by bench.py's CPU baseline and by the
package build step (building the checker is not using it)."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "orc.c")
OUT = os.path.join(HERE, "_build", "liborc.so")


def build(force=False):
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    base = [cc, "-O3", "-fPIC", "-shared", "-std=c11", SRC, "-o", tmp, "-lm"]
    r = subprocess.run(base[:2] + ["-fopenmp"] + base[2:], capture_output=True, text=True)
    if r.returncode != 0:  # no OpenMP runtime: the same loops, serial
        r = subprocess.run(base, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle C build failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
