"""Builds libbeargb300.so in-tree for sm_103a (GB300).

Translation units are compiled in parallel, each with one -gencode; the library
links the shared CUDA runtime so that it shares the runtime with PyTorch when
both are loaded.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbeargb300.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the engine needs the CUDA toolkit to build")
    return p


def _units():
    nv = _nvcc()
    common_cu = [nv, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                 "-Xptxas", "-v", "-I", INCLUDE, "-I", CSRC]
    common_cpp = [nv, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    return [
        ("engine.cu", common_cu),
        ("adjoint.cu", common_cu),
        ("adjoint_transmission.cu", common_cu),
        ("noalloc.cu", common_cu),
        ("priors.cu", common_cu),
        ("contribution.cu", common_cu),
        # bit-faithful host-style arithmetic: no FMA contraction
        ("atmosphere.cu", common_cu + ["--fmad=false"]),
        ("model_setup.cpp", common_cpp + ["-Xcompiler", "-ffp-contract=off"]),
        ("capi.cpp", common_cpp),
    ]


def _sources_digest() -> str:
    h = hashlib.sha1()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cuh", ".cpp", ".h")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode())
                    h.update(fh.read())
    h.update(GENCODE.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the engine if its sources changed; returns the library path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "digest")
    digest = _sources_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    jobs = []
    for src, cmd in _units():
        obj = os.path.join(OUT_DIR, src + ".o")
        jobs.append((obj, cmd + ["-c", os.path.join(CSRC, src), "-o", obj]))

    def run(job):
        obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(run, jobs))
    with open(os.path.join(OUT_DIR, "ptxas.log"), "w") as f:
        for obj, err in results:
            f.write(f"== {os.path.basename(obj)}\n{err}\n")
    if verbose:
        for _, err in results:
            sys.stdout.write(err)
    tmp = LIB + ".tmp"
    link = [_nvcc(), "-shared", GENCODE, "-cudart", "shared", "-o", tmp] + [o for o, _ in results]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
