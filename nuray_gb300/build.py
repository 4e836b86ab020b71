"""Builds libnuray_gpu.so in-tree (nuray_gb300/_build/) with nvcc for sm_103a.

Every translation unit of csrc/ compiled in parallel (CUDA kernels with
nvcc, host C++ with g++), linked with nvcc into one shared library whose
only interface is include/nuray.h. Host code is compiled with
-ffp-contract=off: g++ otherwise fuses a*b + c into FMAs for C++ on
aarch64, and the host arithmetic that must reproduce the reference (SAH
costs, camera, emitter areas) would round differently from x86.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnuray_gpu.so")
CLI = os.path.join(OUT, "nuray")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH") or "/usr/local/cuda"
    return home


def _nvcc():
    return os.path.join(_cuda_home(), "bin", "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def sources():
    out = []
    for d in (CSRC, os.path.join(CSRC, "cli")):
        out += [os.path.join(d, f) for f in sorted(os.listdir(d)) if f.endswith((".cu", ".cpp", ".h", ".cuh"))]
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = sources() + [os.path.join(HERE, "..", "include", h) for h in ("nuray.h", "nuray_renderer.hpp")]
    deps.append(os.path.abspath(__file__))
    return os.path.exists(CLI) and all(os.path.getmtime(p) <= t for p in deps)


def build(force=False, verbose=False):
    """Compiles the library if any source is newer; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "..", "include"), "-I", CSRC]
    cuda_inc = ["-I", os.path.join(_cuda_home(), "include")]
    jobs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        if f.endswith(".cu"):
            jobs.append((obj, [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                               "-Xptxas", "-v" if verbose else "-O3", *inc, "-c", src, "-o", obj]))
        elif f.endswith(".cpp"):
            jobs.append((obj, ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                               *inc, *cuda_inc, "-c", src, "-o", obj]))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    tmp = LIB + ".tmp"
    _run([_nvcc(), *ARCH, "-shared", "-o", tmp, *[j[0] for j in jobs], "-lpthread"])
    os.replace(tmp, LIB)
    # the command-line front end, linked against the library
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", *inc, os.path.join(CSRC, "cli", "nuray_main.cpp"), "-o", CLI,
          "-L", OUT, "-lnuray_gpu", "-Wl,-rpath,$ORIGIN", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
