"""Build ``libhis_gb300.so`` in-tree for sm_103a (GB300) with plain nvcc.

Each translation unit compiles in parallel; the float64 kernels and the 1-D
network are built with ``-fmad=false`` (products and sums round separately, as in
the reference's float64 arithmetic), the float32 kernels with fused multiply-add.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libhis_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
          "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]
UNITS = {
    "capi.cu": [],
    "swe2d_f64.cu": ["-fmad=false"],
    "swe2d_f32.cu": ["-fmad=true", "--use_fast_math"],
    "net1d.cu": ["-fmad=false"],
    "net1d_f32.cu": ["-fmad=true", "--use_fast_math"],
    "noalloc.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhis_gb300.so")


def _sources_digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) +
                    list(INCLUDE.glob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH + COMMON).encode())
    for k, v in UNITS.items():
        h.update((k + " ".join(v)).encode())
    return h.hexdigest()[:16]


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    digest = _sources_digest()
    stamp = BUILD / "digest.txt"
    if LIB.exists() and not force and stamp.exists() and stamp.read_text().strip() == digest:
        return LIB
    cc = nvcc()

    def compile_unit(name: str) -> Path:
        obj = BUILD / (name + ".o")
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], "-c", str(CSRC / name), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = BUILD / f".libhis_gb300.{os.getpid()}.so"
    cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
