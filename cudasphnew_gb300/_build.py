"""Build recipe of the in-tree shared library libsph_gb300.so (sm_103a only).

Each .cu translation unit is compiled in parallel with nvcc, then linked into
cudasphnew_gb300/_build/libsph_gb300.so.  No CMake, no torch extension
machinery: the library is plain C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libsph_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra flags: the boundary-map builder forms every value one rounded
# operation at a time (no FMA contraction), as the reference's host code does.
EXTRA = {"sph_maps.cu": ["--fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OUT, src.replace(".cu", ".o"))
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "-c", os.path.join(CSRC, src), "-o", obj]
    cmd += EXTRA.get(src, [])
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        print(r.stderr)
    return obj


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    if not force and os.path.exists(LIB):
        lib_t = os.path.getmtime(LIB)
        deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
        deps.append(os.path.join(PKG, "..", "include", "sph.h"))
        if all(os.path.getmtime(d) <= lib_t for d in deps if os.path.exists(d)):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose_ptxas="-v" in sys.argv, force=True))
