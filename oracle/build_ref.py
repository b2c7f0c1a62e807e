"""Compile parts of the reference from its own sources, in place, into
oracle/_ref/ (git-ignored).  ORACLE: test infrastructure only.

  oracle/_ref/libpraxis_ref.so   CUDA/praxis.cpp (+ oracle/praxis_ref_shim.cpp)

Runs only where the reference checkout exists (this needs REFERENCE_DIR or the
default checkout path); elsewhere it does nothing and the tests that use its
output skip.  The reference's CUDA programs are not built here: their binaries
would not run on the Arm GPU machine and their sources are not present there.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("REFERENCE_DIR", "/root/reference")


def build():
    src = os.path.join(REF, "CUDA", "praxis.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libpraxis_ref.so")
    shim = os.path.join(HERE, "praxis_ref_shim.cpp")
    if os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(src),
                                                           os.path.getmtime(shim)):
        return lib
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-w", "-o", lib, src, shim]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference praxis build failed:\n" + r.stderr)
    return lib


if __name__ == "__main__":
    print(build())
