"""TEST INFRASTRUCTURE ONLY -- build recipe of the CPU oracle (oracle/_build/liboracle.so).

The oracle is plain C++17 compiled with g++ -O3 and -ffp-contract=off (no FMA contraction, no fast math),
so its single-precision arithmetic follows the source order on x86-64 and aarch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.cpp")]
HEADERS = [os.path.join(HERE, "oracle.h"), os.path.join(ROOT, "include", "spk.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS)


def build(force: bool = False) -> str:
    """Compiles liboracle.so if it is missing or older than its sources; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), *SOURCES, "-o", LIB + ".tmp", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
