"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles oracle/oracle.cpp into oracle/_build/<machine>/liboracle.so with g++ -O3.
`-ffp-contract=off` keeps a*b+c as two roundings, as Rust evaluates it (GCC on
aarch64 would otherwise fuse it into an FMA and change the last bit).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")

FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", *FLAGS, SRC, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
