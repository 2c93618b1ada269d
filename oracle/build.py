"""Build recipe for the CPU oracle (test infrastructure; see nb_oracle.cpp).

``build_oracle()`` compiles ``oracle/nb_oracle.cpp`` and ``oracle/bc6h.cpp`` into ``oracle/_build/libnboracle.so``
with the host compiler.  The flags pin the arithmetic contract: no floating-point
contraction (GCC contracts by default on aarch64), no fast-math.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libnboracle.so")
SOURCES = [os.path.join(HERE, "nb_oracle.cpp"), os.path.join(HERE, "bc6h.cpp"), os.path.join(HERE, "joe_kuo_68.inc")]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
            "-fno-fast-math", "-fno-strict-aliasing", "-Wall", "-Wno-unused-function"]


def build_oracle(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_m for s in SOURCES):
            return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    cmd = [os.environ.get("CXX", "g++"), *CXXFLAGS, "-o", tmp, *[f for f in SOURCES if f.endswith(".cpp")]]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_oracle(force=True))
