"""Build the CPU oracles into oracle/_build/liboracle.so.

ORACLE: test infrastructure only.  Compiled with FMA contraction off and no
fast-math, so the FP32 twin performs exactly the operations written in it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["ismc_twin.c", "ismc_ref64.c"]
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fno-math-errno",
          "-D_GNU_SOURCE", "-Wall", "-Wno-unused-function"]


def build():
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(os.path.dirname(HERE), "include", "ismc.h"), __file__]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["gcc", "-shared", "-o", LIB] + CFLAGS + srcs + ["-lm", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build())
