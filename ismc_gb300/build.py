"""In-tree build of the native libraries of the package.

    python -m ismc_gb300.build            # builds ismc_gb300/libismc.so and the
                                          # command-line programs in ismc_gb300/bin/

Every CUDA translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library next to this file.  FMA contraction is off on
both the device (-fmad=false) and host (-ffp-contract=off) side: the kernels
write every fused multiply-add explicitly, which keeps each packet trajectory
a fixed sequence of correctly rounded operations.  The surrogate network's
unit (ismc_mlp.cu) has no bit-exact CPU twin and is compiled with nvcc's
default contraction.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libismc.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include")] + ARCH

# translation units without a bit-exact CPU restatement: FMA contraction allowed
CONTRACTED = {"ismc_mlp.cu"}
SOURCES = ["ismc_kernels.cu", "ismc_capi.cu", "ismc_noalloc.cu", "ismc_mlp.cu", "ismc_table.cu",
           "ismc_praxis.cpp", "ismc_solve.cpp"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I" + os.path.join(ROOT, "include")]
BIN = os.path.join(HERE, "bin")
# drop-ins for the reference's compiled programs, under the names its drivers
# are pointed at (--CUDAsource .../Lookup.o, .../minimize.o)
PROGRAMS = {"Lookup.o": "cli/cli_lookup.cpp", "minimize.o": "cli/cli_minimize.cpp"}


def nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "ismc.h")]


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    if _newer(obj, [srcp, __file__] + _headers()) and not verbose_ptxas:
        return obj, ""
    if src.endswith(".cpp"):
        cmd = [os.environ.get("CXX", "g++"), "-c", srcp, "-o", obj] + CXX_FLAGS
    else:
        flags = NVCC_FLAGS
        if src in CONTRACTED:
            flags = [f for f in flags if f != "-fmad=false"]
        cmd = [nvcc(), "-c", srcp, "-o", obj] + flags
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stdout + r.stderr


def build(verbose_ptxas=False, quiet=True):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in res]
    logs = "".join(l for _, l in res)
    if not _newer(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart", "-lstdc++"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.makedirs(BIN, exist_ok=True)
    for exe, src in PROGRAMS.items():
        target, srcp = os.path.join(BIN, exe), os.path.join(CSRC, src)
        if _newer(target, [srcp, os.path.join(CSRC, "cli", "cli_common.h"), LIB, __file__]
                  + _headers()):
            continue
        cmd = [os.environ.get("CXX", "g++"), srcp, "-o", target, "-O2", "-std=c++17", "-Wall",
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CSRC, "cli"),
               "-L" + HERE, "-lismc", "-Wl,-rpath,$ORIGIN/..", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of {exe} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if logs and not quiet:
        print(logs)
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, quiet=False))
