"""In-tree build of libgcfd.so for sm_103a (GB300).

Each translation unit is compiled in parallel with nvcc, then linked into
``gocfd_gb300/libgcfd.so`` (CUDA runtime linked statically so the library
loads without an rpath).  The kernels of each polynomial order N = 0..4 sit in
their own units (``gcfd_order.cu`` and ``gcfd_order_adj.cu`` compiled with
-DGCFD_ORDER=N), so the build runs as wide as the host has cores.  No cmake,
no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libgcfd.so")

# (source, extra defines): the per-order units once per order, largest first.
SOURCES = ([("gcfd_order.cu", [f"-DGCFD_ORDER={n}"]) for n in (4, 3, 2, 1, 0)] +
           [("gcfd_order_adj.cu", [f"-DGCFD_ORDER={n}"]) for n in (4, 3, 2, 1, 0)] +
           [("gcfd.cu", []), ("gcfd_adjoint_api.cu", []), ("gcfd_static.cu", []), ("gcfd_post.cu", []), ("gcfd_graph.cu", []), ("gcfd_geometry.cu", []),
            ("gcfd_peaks.cu", []),
            ("dfr_element.cpp", []), ("mesh.cpp", [])])
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgcfd")


def _compile(unit, verbose: bool, extra: list[str]) -> str:
    src, defs = unit
    tag = "".join("_" + d.split("=")[-1] for d in defs)
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + tag + ".o")
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *defs, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr, file=sys.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    hdr = os.path.join(os.path.dirname(PKG_DIR), "include", "gcfd.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile libgcfd.so if any source is newer than it; return its path."""
    if not force and not ptxas_info and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    workers = max(1, min(len(SOURCES), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose or ptxas_info, extra), SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          ptxas_info="--ptxas" in sys.argv)
    print(LIB_PATH)
