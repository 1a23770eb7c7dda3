"""Build libcp3gb300.so in-tree (cudaprob3_gb300/_lib/) with nvcc for sm_103a.

Translation units compile in parallel; cp3_tables.cu (the FP64 eigen work that mirrors the
reference's arithmetic) is compiled without FMA contraction, everything else with it.
``python -m cudaprob3_gb300.build`` or ``cudaprob3_gb300.build.build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libcp3gb300.so")
PEAKS_LIB = os.path.join(OUT, "libcp3peaks.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags).  The host geometry and parameter code is compiled without FMA
# contraction (aarch64 compilers contract by default): grazing trajectories turn one-ulp
# differences of r^2 - R^2 (1 - cos^2) into centimetre changes of a segment, and the FP64
# path is meant to see the same segment lengths as the reference's build.
UNITS = [
    ("cp3_host.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("cp3_abi.cu", []),
    ("cp3_tables.cu", ["-fmad=false"]),
    ("cp3_atmos.cu", []),
    ("cp3_noalloc.cu", []),
    ("cp3_batch.cu", []),
    ("cp3_serve.cu", []),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcp3gb300.so")


def _sources_mtime() -> float:
    newest = 0.0
    for root in (SRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(root):
            newest = max(newest, os.path.getmtime(os.path.join(root, f)))
    return newest


# The debug build: the same library with the persistent kernel's arena bounds checks
# compiled in (-DCP3_DEVICE_CHECKS).  A tile whose accesses would leave an arena is skipped
# and reported as a status; select it at run time with CP3GB300_LIB=<this path>.
OUT_CHECKED = os.path.join(OUT, "checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libcp3gb300.so")


def _signature(nvcc, common, device_checks) -> str:
    """Digest of everything besides the sources that decides the library's contents: the
    compiler, the target, the common flags and every unit's own flags (cp3_tables.cu's
    -fmad=false is what keeps the FP64 masses on the reference's roundings)."""
    import hashlib
    import json
    text = json.dumps([os.path.realpath(nvcc), ARCH, [c for c in common if c != "-v"], UNITS,
                       bool(device_checks)])
    return hashlib.sha256(text.encode()).hexdigest()


def build(force: bool = False, verbose: bool = False, device_checks: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library (the debug build with
    device bounds checks when device_checks is set).  The library is stale when a source or
    header is newer than it, or when the compile commands differ from the ones it was built
    with (recorded beside it in build.sig)."""
    out, lib = (OUT_CHECKED, LIB_CHECKED) if device_checks else (OUT, LIB)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", SRC,
              "-I", os.path.join(os.path.dirname(HERE), "include")]
    if device_checks:
        common += ["-DCP3_DEVICE_CHECKS"]
    sig = _signature(nvcc, common, device_checks)
    sig_path = os.path.join(out, "build.sig")
    try:
        with open(sig_path) as f:
            same_commands = f.read().strip() == sig
    except OSError:
        same_commands = False
    if (not force and same_commands and os.path.exists(lib)
            and os.path.getmtime(lib) >= _sources_mtime()):
        return lib
    os.makedirs(out, exist_ok=True)
    if os.path.exists(sig_path):
        os.remove(sig_path)  # a build that fails half-way leaves no signature behind
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(unit):
        src, extra = unit
        obj = os.path.join(out, src.rsplit(".", 1)[0] + ".o")
        cmd = [nvcc] + ARCH + common + extra + ["-c", os.path.join(SRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return obj, r, cmd

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_one, UNITS))
    logs = []
    for obj, r, cmd in results:
        logs.append(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    tmp = lib + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + [o for o, _, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)
    if device_checks:
        with open(sig_path, "w") as f:
            f.write(sig)
        return lib
    # bench support: scalar FMA peaks (separate library, not part of the C ABI)
    cmd = [nvcc] + ARCH + common + ["-shared", os.path.join(SRC, "cp3_peaks.cu"), "-o", PEAKS_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    with open(os.path.join(OUT, "build.log"), "w") as f:
        f.write("\n".join(logs))
    with open(sig_path, "w") as f:
        f.write(sig)
    if verbose:
        sys.stdout.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                device_checks="--device-checks" in sys.argv))
