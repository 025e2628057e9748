"""Build libpn_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel (`nvcc -c`), then linked with
`nvcc -shared`.  Host code is compiled with -ffp-contract=off so that the geometry
computed on the host (padded corners, periodic cell sizes) is rounded like the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpn_gb300.so")
# the bounds-checked variant (-DPN_BOUNDS_CHECK), built on request into its own folder
BC_DIR = os.path.join(OUT_DIR, "bounds_check")
LIB_BC = os.path.join(OUT_DIR, "libpn_gb300_bc.so")
SOURCES = ["pn_api.cu", "pn_build.cu", "pn_traverse_f32.cu", "pn_traverse_f64.cu",
           "pn_traverse_mixed.cu", "pn_traverse_mixed_lists.cu", "pn_traverse_f32_sph.cu",
           "pn_traverse_f64_sph.cu", "pn_traverse_mixed_sph.cu", "pn_noalloc.cu",
           "pn_batch.cu", "pn_precomputed.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpn_gb300")


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "pn_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(f) > t for f in _deps())


def _compile(src: str, verbose_ptxas: bool, bounds_check: bool = False) -> str:
    out = BC_DIR if bounds_check else OUT_DIR
    obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), "-c",
           os.path.join(CSRC, src), "-o", obj]
    if bounds_check:
        cmd[1:1] = ["-DPN_BOUNDS_CHECK"]
    if verbose_ptxas:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, bounds_check: bool = False) -> str:
    """Compile the library if any source changed; return its path.  bounds_check: the
    variant that checks every device index (libpn_gb300_bc.so, PN_BOUNDS_CHECK)."""
    lib = LIB_BC if bounds_check else LIB
    if not force and not stale(lib):
        return lib
    os.makedirs(BC_DIR if bounds_check else OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas, bounds_check), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl",
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv,
                bounds_check="--bounds-check" in sys.argv))
