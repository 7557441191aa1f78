"""Builds the native libraries in-tree: fastbact_gb300/_lib/libfbk.so (the device
path and its host side) and fastbact_gb300/_lib/libfbk_synth.so (the seeded input
generator, a host-only library of its own so that a CPU-only caller generating
workloads never maps the device library).

CUDA translation units are compiled for sm_103a only; host C++ units with g++.
-ffp-contract=off keeps the estimator's f64 host arithmetic free of fused
multiply-adds (Arm compilers contract by default), so it rounds like the
reference's Rust f64 code.  Units compile in parallel; an unchanged source set
is not rebuilt (a hash of sources and flags is stored next to the library).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libfbk.so"
SYNTH_LIB = LIB_DIR / "libfbk_synth.so"
BUILD_DIR = ROOT / "_build" / "fbk"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-pthread"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastbact_gb300")


def sources() -> tuple[list[Path], list[Path]]:
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    return cu, cpp


def synth_sources() -> list[Path]:
    """The generator plus the host ingest it runs to make a read bank."""
    return sorted((CSRC / "synth").glob("*.cpp")) + [CSRC / "host" / "fbk_ingest.cpp", CSRC / "host" / "fbk_workers.cpp"]


def _digest(files: list[Path]) -> str:
    h = hashlib.sha256()
    for f in sorted(files):
        h.update(f.name.encode())
        h.update(f.read_bytes())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> Path:
    cu, cpp = sources()
    synth = synth_sources()
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((CSRC / "host").glob("*.h")) + list(
        (ROOT / "include").glob("*.h"))
    digest = _digest(cu + cpp + synth + headers)
    stamp = LIB_DIR / "libfbk.sha256"
    if (not force and LIB.exists() and SYNTH_LIB.exists() and stamp.exists()
            and stamp.read_text().strip() == digest):
        return LIB
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    for src in cu:
        obj = BUILD_DIR / (src.stem + ".o")
        jobs.append([nvcc, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD_DIR / (src.stem + ".o")
        jobs.append([cxx, *CXX_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])
    synth_tmp = LIB_DIR / "libfbk_synth.so.tmp"
    # -Bsymbolic: the generator's own copy of the host ingest binds to itself even
    # when libfbk.so (which exports the same ingest entry points) is loaded first
    jobs.append([cxx, *CXX_FLAGS, "-shared", "-Wl,--no-undefined", "-Wl,-Bsymbolic", "-I", str(ROOT / "include"),
                 *[str(s) for s in synth], "-o", str(synth_tmp)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out, file=sys.stderr)
    objs = [str(BUILD_DIR / (s.stem + ".o")) for s in cu + cpp]
    tmp = LIB_DIR / "libfbk.so.tmp"
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lpthread"])
    os.replace(tmp, LIB)
    os.replace(synth_tmp, SYNTH_LIB)
    stamp.write_text(digest)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
