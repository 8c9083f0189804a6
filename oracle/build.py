"""Build recipe of the oracle (test infrastructure): g++ -O2 -ffp-contract=off
(no fast-math, no FMA contraction) so every float expression is evaluated as
the written sequence of IEEE binary32 operations.  Output: oracle/_build/liboracle.so
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle.so")


def build():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-math-errno", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-o", tmp, os.path.join(HERE, "vrg_oracle.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build())
