"""Builds libnxm_cuda.so in the package directory with nvcc for sm_103a.

Each translation unit is compiled separately (in parallel) into _build/,
then linked into nexusmd_gb300/libnxm_cuda.so.  Only files whose sources or
headers changed are recompiled.  Host-only C++ goes through nvcc too, so the
same compiler and flags are used on x86 and on Arm hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libnxm_cuda.so")
# bench-only hardware probes (FP32 FMA peak, shared-memory atomics): a library
# of their own beside bench.py, outside the engine and its C ABI
PROBE_SRC = os.path.join(ROOT, "bench_probe.cu")
PROBE_LIB = os.path.join(ROOT, "libnxm_probe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["k_neighbor.cu", "k_pairs.cu", "k_bonded.cu", "k_nonbonded.cu", "k_fft.cu", "k_pme.cu",
                "k_integrate.cu", "nxm_engine.cu", "nxm_abi.cpp", "nxm_dispatcher.cpp", "k_pme_noalloc.cu",
                "nxm_report.cpp", "k_exclusions_build.cu"]
HOST_SOURCES = ["nxm_xml.cpp", "nxm_io.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers_digest() -> str:
    h = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                    + glob.glob(os.path.join(ROOT, "include", "*.h"))):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _compile(src: str, extra: list[str], hdr: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    stamp = obj + ".stamp"
    with open(path, "rb") as f:
        key = hashlib.sha256(f.read() + hdr.encode() + " ".join(extra).encode()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj
    # -ffp-contract=off: host FP64 set-up code (box, moduli, influence
    # function) must round like the reference's unfused x86 build on Arm too
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                             "-Xcompiler", "-ffp-contract=off",
                             "-I" + CSRC, "-I" + os.path.join(ROOT, "include")] + extra + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-8000:]))
    with open(stamp, "w") as f:
        f.write(key)
    return obj


def build(verbose: bool = False) -> str:
    """Compile and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_digest()
    jobs = [(s, ["-x", "cu"] if s.endswith(".cpp") else []) for s in CUDA_SOURCES]
    jobs += [(s, ["-x", "c++"]) for s in HOST_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(j[0], j[1], hdr), jobs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    build_probe(verbose)
    return LIB


def build_probe(verbose: bool = False) -> str:
    """Compile bench_probe.cu into libnxm_probe.so (bench.py's hardware probes)."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "probe.stamp")
    with open(PROBE_SRC, "rb") as f:
        key = hashlib.sha256(f.read()).hexdigest()
    if os.path.exists(PROBE_LIB) and os.path.exists(stamp) and open(stamp).read() == key:
        return PROBE_LIB
    tmp = PROBE_LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                             PROBE_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for bench_probe.cu:\n" + r.stderr[-4000:])
    os.replace(tmp, PROBE_LIB)
    with open(stamp, "w") as f:
        f.write(key)
    if verbose:
        print("built", PROBE_LIB)
    return PROBE_LIB


if __name__ == "__main__":
    build(verbose=True)
