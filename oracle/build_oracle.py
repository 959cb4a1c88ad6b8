"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Compiles oracle/chflow_oracle.c into oracle/_build/liboracle.so with gcc.
-ffp-contract=off keeps x86 and Arm hosts on identical rounding.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "chflow_oracle.c")
    hdr = os.path.join(HERE, "chflow_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
