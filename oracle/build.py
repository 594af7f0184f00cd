"""Build recipe for the oracle library (test infrastructure; no reference sources are compiled).

``liboracle.so`` is built from ``fem2d_oracle.cpp`` with g++ only, without fused multiply-adds (the
reference's Rust arithmetic rounds every product and sum). It is rebuilt on the machine that
runs the tests, since nothing compiled on one architecture runs on the other.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_oracle(force=False):
    src = os.path.join(HERE, "fem2d_oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-Wall", "-Wno-unused-function",
           "-Wno-psabi",   # GCC's note on aarch64 that std::pair argument passing changed in GCC 10
           src, "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
