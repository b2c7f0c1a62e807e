"""Build parts of the reference from its own sources into oracle/_ref/
(git-ignored).  ORACLE / baseline infrastructure only.

  oracle/_ref/libpraxis_ref.so   CUDA/praxis.cpp (+ oracle/praxis_ref_shim.cpp),
                                 compiled in place where the reference checkout
                                 exists; tests compare the project's PRAXIS with it
  oracle/_ref/src/CUDAISMLMC.h   a byte-for-byte copy of the reference's CUDA
                                 forward model (CUDA/CUDAISMLMC.h), staged here
                                 so that it travels with the working tree to the
                                 GPU machine, where the reference checkout is
                                 absent.  It is never committed (oracle/_ref/ is
                                 git-ignored) and never edited.
  oracle/_ref/drivers/           byte-for-byte copies of the reference's driver
                                 scripts and their example configurations
                                 (Lookup/lookup.py, Minimization/minimization.py,
                                 */example.ini), staged the same way for the
                                 end-to-end driver tests on the GPU machine
  oracle/_ref/python/            byte-for-byte copies of the reference's Python
                                 forward model (ISMLMC.py, MLMC.py), staged the
                                 same way, so that the reference itself can be
                                 timed on the GPU machine's host cores
                                 (oracle/refpython.py)
  oracle/_ref/refcuda_bench      oracle/refcuda_bench.cu, the project's timing
                                 harness, compiled against the staged header
                                 for sm_103a (build_refcuda(), on the GPU
                                 machine, on demand)

The reference checkout is found through REFERENCE_DIR, else at its usual
location in the build container; where neither exists, the in-place builds are
skipped and whatever was staged earlier is used.
"""
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
DEFAULT_REFERENCE_DIR = "/root/reference"
# the reference's CUDA forward model: kernel CUDAISMLMC (CUDAISMLMC.h:316-654)
# and its host wrapper ISMLMC() (CUDAISMLMC.h:656-755)
STAGED = ("CUDA/CUDAISMLMC.h",)
# the reference's driver scripts (run unmodified through ismc_gb300.dropin.drivers)
DRIVERS = ("Lookup/lookup.py", "Lookup/example.ini", "Minimization/minimization.py",
           "Minimization/example.ini")
DRIVERS_DIR = os.path.join(OUT, "drivers")
# the reference's Python forward model: ISMLMC() (ISMLMC.py:101-347) and the
# multilayer walk it calls (MLMC.py:283-409); it imports only math and random
PYTHON_MODEL = ("ISMLMC.py", "MLMC.py")
PYTHON_DIR = os.path.join(OUT, "python")
HARNESS = os.path.join(HERE, "refcuda_bench.cu")
REFCUDA_BIN = os.path.join(OUT, "refcuda_bench")


def reference_dir():
    """The reference checkout, or None where it is absent."""
    d = os.environ.get("REFERENCE_DIR", DEFAULT_REFERENCE_DIR)
    return d if os.path.isdir(d) else None


def _sha(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def stage():
    """Copy the reference's CUDA forward model, its driver scripts and its
    Python forward model, unmodified, into oracle/_ref/ (src/, drivers/, python/).
    Returns the staged header's path, or None when neither the checkout nor an
    earlier staged copy exists."""
    ref = reference_dir()
    if ref:
        copies = [(rel, os.path.join(SRC, os.path.basename(rel))) for rel in STAGED]
        copies += [(rel, os.path.join(DRIVERS_DIR, rel)) for rel in DRIVERS]
        copies += [(rel, os.path.join(PYTHON_DIR, rel)) for rel in PYTHON_MODEL]
        for rel, dst in copies:
            src = os.path.join(ref, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            if not os.path.exists(dst) or _sha(dst) != _sha(src):
                shutil.copyfile(src, dst)
    hdr = os.path.join(SRC, "CUDAISMLMC.h")
    return hdr if os.path.exists(hdr) else None


def staged_driver(rel):
    """Path of a staged reference driver file (e.g. "Minimization/minimization.py"),
    or None where it was never staged."""
    stage()
    p = os.path.join(DRIVERS_DIR, rel)
    return p if os.path.exists(p) else None


def staged_python():
    """Directory holding the staged ISMLMC.py / MLMC.py, or None where they
    were never staged."""
    stage()
    ok = all(os.path.exists(os.path.join(PYTHON_DIR, f)) for f in PYTHON_MODEL)
    return PYTHON_DIR if ok else None


def build_praxis():
    ref = reference_dir()
    if not ref:
        return None
    src = os.path.join(ref, "CUDA", "praxis.cpp")
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


def build_refcuda():
    """Compile the timing harness against the staged reference header for
    sm_103a.  The only change to the reference's build is -DclockRate=major:
    CUDA 13 removed cudaDeviceProp::clockRate, which the reference's
    CUDABasicProperties() (CUDAISMLMC.h:29-39, never called by the harness)
    prints.  Returns the binary's path, or None without a staged header."""
    hdr = stage()
    if not hdr:
        return None
    if os.path.exists(REFCUDA_BIN) and os.path.getmtime(REFCUDA_BIN) >= max(
            os.path.getmtime(hdr), os.path.getmtime(HARNESS)):
        return REFCUDA_BIN
    nvcc = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    cmd = [nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
           "-DclockRate=major", "-w", "-I" + SRC, HARNESS, "-o", REFCUDA_BIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference CUDA harness build failed:\n" + " ".join(cmd) + "\n" +
                           r.stdout + r.stderr)
    return REFCUDA_BIN


def build():
    """What build() of the project does with the reference: the in-place PRAXIS
    library and the staged CUDA header (no CUDA compilation here)."""
    stage()
    return build_praxis()


if __name__ == "__main__":
    print(build())
    print(stage())
