"""Compiles oracle/heal_oracle.c into oracle/liboracle.so (gcc, OpenMP)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "heal_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    hdr = os.path.join(HERE, "..", "include", "heal_gb300.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-fopenmp", "-fPIC", "-shared", "-Wall",
           SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
