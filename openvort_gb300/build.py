"""Build libovgpu.so (CUDA, sm_103a) in-tree with nvcc.

    python -m openvort_gb300.build

Translation units compile in parallel into openvort_gb300/lib/_obj and link
into openvort_gb300/lib/libovgpu.so.  Host code is compiled with
-ffp-contract=off so the few host-side FP64 steps (parameter normalisation,
geometry) round the same on x86 and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "_obj")
SO = os.path.join(LIB, "libovgpu.so")
DROPIN = os.path.join(LIB, "libovdropin.a")

CU_SOURCES = ["ov_sort.cu", "ov_tree.cu", "ov_velocity.cu", "ov_capi.cu", "ov_topology.cu", "ov_peak.cu",
              "ov_frames.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libovgpu")


def _compile(src: str, verbose: bool) -> tuple[str, str]:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{p.stderr}")
    return obj, p.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    newest = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= newest:
        return SO
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = SO + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stderr}")
    os.replace(tmp, SO)
    build_dropin()
    return SO


def build_dropin() -> str:
    """ov_dropin.c -> libovdropin.a (with the __wrap_ aliases) for linking into the reference."""
    cc = shutil.which("gcc") or shutil.which("cc")
    obj = os.path.join(OBJ, "ov_dropin.o")
    subprocess.run([cc, "-O2", "-fPIC", "-ffp-contract=off", "-DOV_DROPIN_WRAP", "-c",
                    os.path.join(CSRC, "ov_dropin.c"), "-o", obj], check=True)
    if os.path.exists(DROPIN):
        os.remove(DROPIN)
    subprocess.run(["ar", "rcs", DROPIN, obj], check=True)
    return DROPIN


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
