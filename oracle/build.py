"""Build the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.

The oracle restates the reference algorithms on the CPU; tests, the smoke check
and the CPU-baseline leg of bench.py load it as the checker.  Compiled without
FMA contraction so float results follow the written evaluation order.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]


def build_oracle() -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, *FLAGS, SRC, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle())
