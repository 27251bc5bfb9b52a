"""Build libqgcore.so in-tree with nvcc for sm_103a (no cmake, no torch extension).

Each translation unit compiles in parallel to an object file under ``somax_gb300/_build``;
they are linked into ``somax_gb300/lib/libqgcore.so`` with the CUDA runtime linked
statically, so the library needs only the driver at run time.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libqgcore.so"
SOURCES = ["qg_plan.cu", "qg_stencil.cu", "qg_gemm_simt.cu", "qg_gemm_tc.cu", "qg_static.cu", "qg_persistent.cu", "qg_adjoint.cu", "qg_sweep.cu", "qg_lsweep.cu", "qg_capacitance.cu", "qg_mask.cu", "qg_cluster.cu", "qg_swm.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libqgcore.so cannot be built")


def _compile(src: pathlib.Path, obj: pathlib.Path, extra: list[str]) -> tuple[str, str]:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
           "-Xptxas", "-v" if os.environ.get("QG_PTXAS_V") else "-O3",
           "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return src.name, r.stderr


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "qgcore.h"]
    newest_hdr = max(h.stat().st_mtime for h in headers)
    jobs = []
    for s in SOURCES:
        src = CSRC / s
        obj = BUILD / (s + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_hdr):
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for name, log in ex.map(lambda a: _compile(a[0], a[1], []), jobs):
            if verbose and log:
                print(f"[{name}]\n{log}", file=sys.stderr)
    objs = [str(BUILD / (s + ".o")) for s in SOURCES]
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "--cudart", "static", "-o", str(tmp), *objs, "-ldl", "-lrt", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
